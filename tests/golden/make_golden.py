"""Regenerates tests/golden/*.json from the reference's own unit tests.

Reads the reference sources as text (nothing is compiled or executed):
  unit_tests/kernel_test.cpp          closed-form W(q) and grad W(q) values
  unit_tests/smoothing_test.cpp       4-particle smoothing, sigma* = 20/(7 pi)
  unit_tests/grad_smoothing_test.cpp  5-particle pressure gradient 45/(8 pi)
  unit_tests/evolver_test.cpp         RK2 with a no-op derivative functional
  unit_tests/eos_interpolator_test.cpp exact multilinear interpolation

Usage: python tests/golden/make_golden.py <path to a CCAKE checkout>
The committed JSON files are what the tests read; the reference is not needed
at test time.
"""
import json
import math
import os
import re
import sys

OUT = os.path.dirname(os.path.abspath(__file__))


def ev(expr, **env):
    expr = expr.replace("M_PI", "math.pi").strip()
    return float(eval(expr, {"math": math, **env}))


H_RE = r"double(?:\s+const)?\s+h\s*=\s*([^;]+);"


def kernel_cases():
    path = os.path.join(REF, "unit_tests", "kernel_test.cpp")
    src = open(path).read()
    cases = []
    for m in re.finditer(r"TEST\(\s*(\w+)\s*,\s*(\w+)\s*\)\s*\{(.*?)\n\}", src, re.S):
        suite, name, body = m.group(1), m.group(2), m.group(3)
        line = src[:m.start()].count("\n") + 1
        if suite == "KernelTest":
            d = ev(re.search(r"double dist\s*=\s*([^;]+);", body).group(1))
            h = ev(re.search(H_RE, body).group(1))
            k = re.search(r"SPHkernel<(\d)>::kernel\(dist,h\)(?:-([^)]*\)?[^,]*?))?\s*\)\s*,\s*TOL", body)
            D = int(k.group(1))
            expect = 0.0 if k.group(2) is None else ev(k.group(2))
            cases.append(dict(kind="W", D=D, r=d, h=h, expect=expect,
                              cite=f"unit_tests/kernel_test.cpp:{line}"))
        elif suite == "GradKernelTest":
            D = int(re.search(r"SPHkernel<(\d)>", body).group(1))
            h = ev(re.search(H_RE, body).group(1))
            tv = ev(re.search(r"target_val\s*=\s*([^;]+);", body).group(1), h=h)
            pa = [ev(x) for x in re.search(r"pos_a\[\d\]\s*=\s*\{([^}]*)\}", body).group(1).split(",")]
            pb = [ev(x) for x in re.search(r"pos_b\[\d\]\s*=\s*\{([^}]*)\}", body).group(1).split(",")]
            rel = [a - b for a, b in zip(pa, pb)]
            expect = [0.0] * D
            axis = max(range(D), key=lambda i: abs(rel[i]))
            expect[axis] = tv
            cases.append(dict(kind="gradW", D=D, rel=rel, h=h, expect=expect,
                              cite=f"unit_tests/kernel_test.cpp:{line}"))
    return cases


def main():
    kc = kernel_cases()
    smoothing = dict(
        cite="unit_tests/smoothing_test.cpp:33-125",
        note="four 2-D particles, h = 1, sph mass 1, extensive 1: sigma_lab(0) = s*(0) = 20/(7 pi)",
        positions=[[0.0, 0.0], [0.0, 0.5], [0.8, 0.6], [1.5, 0.0]],
        h=1.0,
        sigma_lab_0=20.0 / (7.0 * math.pi),
    )
    gradient = dict(
        cite="unit_tests/grad_smoothing_test.cpp:26-70",
        note="five 2-D particles, p = 1, .5, 1.5, 2.5, 1 and sigma_lab = 1, h = 1: dP/dx(0) = 45/(8 pi), dP/dy(0) = 0",
        positions=[[0.0, 0.0], [0.5, 0.0], [1.0, 0.0], [1.5, 0.0], [-1.5, 1.5]],
        p=[1.0, 0.5, 1.5, 2.5, 1.0],
        h=1.0,
        gradP_0=[45.0 / (8.0 * math.pi), 0.0],
    )
    with open(os.path.join(OUT, "kernel_golden.json"), "w") as f:
        json.dump(dict(source="unit_tests/kernel_test.cpp", tol=1e-14, cases=kc), f, indent=1)
    with open(os.path.join(OUT, "sph_sums_golden.json"), "w") as f:
        json.dump(dict(smoothing=smoothing, gradient=gradient), f, indent=1)
    print(f"{len(kc)} kernel cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    REF = sys.argv[1]
    main()
