"""The diffusion sector in the mixed form against the FP64 oracle.

The mixed form with the sector: FP32 Kahan pair sums (smoothing, gradients
and the diffusion sums of src/sph_workstation.cpp:909-967), FP32 equations
of motion including the diffusion MRFs (src/eom_default.cpp:1415-1817); FP64
EoS inversion and alpha derivatives, q^mu reconstruction and regulator, and
the RK2 update of the state and of the extensive currents. Bar: 1e-5
relative in e and the charge densities after the steps run (the mixed form's
bar), the currents q^mu within 1e-4 of their own range.
"""
import dataclasses

import numpy as np
import pytest

from ccake_gb300 import api, ics
import oracle_py as O

pytestmark = pytest.mark.gpu

KAPPA = (0.3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.3)


def relerr_big(a, b, frac=1e-3):
    # relative error where |b| is at least frac of the field's largest magnitude
    m = np.abs(b) >= frac * np.max(np.abs(b))
    return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m])))


def relerr_range(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def case(name):
    if name == "hotspots2d":
        p, rc = ics.hotspots_2d(n_side=40, n_hot=5, seed=11)
        return p, dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=KAPPA), None, 20
    if name == "hotspots3d":
        p, rc = ics.hotspots_3d(n_xy=16, n_eta=12, n_hot=4, seed=3)
        return p, dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=KAPPA), None, 8
    # baryon only, conformal EoS, kappa_B from the coth form, the regulator on
    # and an initial current part of which it caps
    p, rc = ics.hotspots_2d(n_side=40, n_hot=5, seed=13)
    p = dataclasses.replace(p, e=50.0 * p.e, rhoB=200.0 * p.rhoB, rhoQ=np.zeros_like(p.rhoQ))
    rc = dataclasses.replace(rc, eos_kind=0, thermo_mode=0, using_diffusion=1, diffusion_mode=2,
                             diffusion_relax_mode=1, C_B=0.4, diffusion_regulator=1)
    q = np.zeros((12, p.n))
    q[1] = 12.0 * p.rhoB * np.cos(6.0 * p.x)
    q[2] = 6.0 * p.rhoB * np.sin(5.0 * p.y)
    return p, rc, q, 20


def run_gpu(p, rc, q, steps):
    g = api.GpuHydro(rc)
    g.load(p)
    if q is not None:
        g.set_initial_diffusion(q)
    g.initialize()
    g.step(steps)
    return g


@pytest.mark.parametrize("name", ["hotspots2d", "hotspots3d", "coth"])
def test_mixed_diffusion_matches_oracle(name):
    p, rc, q, steps = case(name)
    orc = O.OracleRun(p, rc)
    if q is not None:
        for c, C in enumerate("BSQ"):
            for m in range(4):
                orc.set(f"in_q{C}{m}", q[4 * c + m])
    assert orc.initialize() == 0
    assert orc.step(steps) == 0
    mixed = run_gpu(p, dataclasses.replace(rc, precision=1), q, steps)
    assert abs(mixed.t - orc.t) < 1e-12
    charges = ("rhoB",) if name == "coth" else ("rhoB", "rhoQ")
    for f in ("e", "s", "T") + charges:
        assert relerr_big(mixed.get(f), orc.get(f)) < 1e-5, f
    for f in (("qB1", "qB2") if name == "coth" else ("qB1", "qB2", "qQ1", "qQ2")):
        # the currents (grown from zero in the hot-spot cases) carry the
        # diffusion MRFs of every step
        assert np.max(np.abs(orc.get(f))) > 0.0, f
        assert relerr_range(mixed.get(f), orc.get(f)) < 1e-4, f


def test_mixed_diffusion_off_matches_mixed_plain():
    # kappa = 0 and no current: the sector leaves the mixed evolution as it is
    p, rc = ics.hotspots_2d(n_side=32, n_hot=4, seed=5)
    rc = dataclasses.replace(rc, precision=1)
    plain = run_gpu(p, rc, None, 5)
    zero = run_gpu(p, dataclasses.replace(rc, using_diffusion=1), None, 5)
    for f in ("x", "u0", "e", "ext_B"):
        assert relerr_range(zero.get(f), plain.get(f)) < 1e-12, f
