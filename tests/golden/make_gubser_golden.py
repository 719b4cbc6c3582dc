"""Extracts the reference's semi-analytic viscous Gubser tables into
tests/golden/gubser_semianalytic.json.

Source: misc/Gubser_checks/ac/*_SemiAnalytic.dat of a CCAKE checkout
(Israel-Stewart Gubser flow, eta/s = 0.2, tau_pi = 5 eta/(e + p), conformal
e = 3p; columns x, y [fm], T [GeV], u^x, u^y, pi^xx, pi^yy, pi^xy,
tau^2 pi^{eta eta} [GeV/fm^3]; the README in that folder). The files are read
as text; every row of the tau = 1 fm/c profile and every second row (x steps
of 0.1 fm) of the later ones are kept.

Usage: python tests/golden/make_gubser_golden.py <path to a CCAKE checkout>
The committed JSON is what the tests read; the reference is not needed at test
time.
"""
import glob
import json
import os
import sys

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gubser_semianalytic.json")
COLUMNS = ["x", "y", "T_GeV", "ux", "uy", "pixx", "piyy", "pixy", "tau2_pietaeta"]


def main(ref):
    folder = os.path.join(ref, "misc", "Gubser_checks", "ac")
    tables = []
    for path in sorted(glob.glob(os.path.join(folder, "*_SemiAnalytic.dat"))):
        name = os.path.basename(path)
        line = name.split("_")[0]                       # "y=0" or "y=x"
        tau = float(name.split("tau=")[1].split("_")[0].rstrip("."))
        rows = []
        with open(path) as fh:
            for ln in fh:
                parts = ln.split()
                if len(parts) == len(COLUMNS):
                    rows.append([float(v) for v in parts])
        if tau != 1.0:
            rows = rows[::2]
        tables.append(dict(file=f"misc/Gubser_checks/ac/{name}", line=line, tau=tau, rows=rows))
    doc = dict(source="misc/Gubser_checks/ac (README.txt: eta/s = 0.2, tau_R = 5 eta/(e+P), e = 3P)",
               columns=COLUMNS, tables=tables)
    with open(OUT, "w") as fh:
        json.dump(doc, fh, separators=(",", ":"))
    print(f"{len(tables)} tables, {sum(len(t['rows']) for t in tables)} rows -> {OUT}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])
