"""The FP64 GPU path on the reference's viscous Gubser check
(misc/Gubser_checks/ac: Israel-Stewart, eta/s = 0.2, tau_pi = 5 eta/w,
conformal EoS), through the C ABI.

* GPU against the oracle at 1e-10 after 50 RK2 steps (141 x 141 lattice).
* GPU against the reference's semi-analytic tables at tau = 1.2, 1.5 and
  2.0 fm/c along y = 0 and y = x, at three resolutions (dx = 0.1, 0.05,
  0.025 fm with h = 2 dx, lattices of 141^2, 281^2 and 561^2 particles over
  [-7, 7]^2 fm, dt = 0.001 fm/c): the error falls as h falls from 0.2 to
  0.1 fm, and at h = 0.1 fm (the reference's run) T stays within 1 %, u
  within 1 % and pi within 5 % of their largest magnitude up to tau = 2 fm/c
  (measured on GB300: at tau = 2, T 0.82 %, u 0.72 %, pi 4.2 %; the T error
  at tau = 2 levels off near 0.8 % as h falls further, a difference between
  the SPH equations and the semi-analytic solution that resolution does not
  remove).
"""
import numpy as np
import pytest

import gubser_tables as GT
import oracle_py as O
from ccake_gb300 import api, ics

pytestmark = pytest.mark.gpu

RES = ((141, 0.1), (281, 0.05), (561, 0.025))
TAUS = (1.2, 1.5, 2.0)


def _gpu(n_side, dx):
    p, rc, pi = ics.gubser_viscous_2d(n_side=n_side, dx=dx, h=2 * dx)
    g = api.GpuHydro(rc)
    g.load(p)
    g.set_initial_viscous(None, pi)
    g.initialize()
    return p, rc, pi, g


def test_viscous_gubser_gpu_matches_oracle():
    p, rc, pi, g = _gpu(141, 0.1)
    orc = O.OracleRun(p, rc)
    orc.set_initial_viscous(None, pi)
    assert orc.initialize() == 0
    g.step(50)
    assert orc.step(50) == 0
    for f in ("x", "y", "u0", "u1", "ext_s", "T", "e", "sigma_lab", "ext_shv0", "ext_shv1", "ext_shv3", "shv11",
              "shv22", "shv12", "shv33", "Ez"):
        a, b = g.get(f), orc.get(f)
        # u^y, u^x and pi^xy vanish on the axes: checked against 1e-5 of their range
        floor = 1e-5 if f in ("u0", "u1", "ext_shv1", "shv12") else 1e-6
        scale = np.abs(b) + floor * np.max(np.abs(b)) + 1e-300
        assert np.max(np.abs(a - b) / scale) < 1e-10, f


@pytest.fixture(scope="module")
def errors():
    tabs = GT.load()
    out = {}
    for n_side, dx in RES:
        _, rc, _, g = _gpu(n_side, dx)
        done = 0
        for tau in TAUS:
            k = int(round((tau - rc.t0) / rc.dt)) - done
            g.step(k)
            done += k
            assert abs(g.t - tau) < 1e-11
            x, y = g.get("x"), g.get("y")
            f = GT.sph_fields(g.get, g.t)
            for line, xlim in (("y=0", 4.5), ("y=x", 3.5)):
                out[(dx, tau, line)] = GT.line_errors(tabs[(line, tau)], line, x, y, f, dx, xlim)
        g.close()
    for key in sorted(out):
        print("gubser IS", key, {k: f"{v:.2e}" for k, v in out[key].items()})
    return out


def test_viscous_gubser_converges_to_reference_tables(errors):
    for tau in TAUS:
        for line in ("y=0", "y=x"):
            e1, e2 = errors[(0.1, tau, line)], errors[(0.05, tau, line)]
            for k in ("T", "ux"):
                assert e2[k] < e1[k], (tau, line, k, e1[k], e2[k])
            pik = [k for k in e1 if k.startswith("pi") or k == "t2pee"]
            assert max(e2[k] for k in pik) < max(e1[k] for k in pik), (tau, line)


def test_viscous_gubser_reference_resolution_within_bounds(errors):
    for tau in TAUS:
        for line in ("y=0", "y=x"):
            e = errors[(0.05, tau, line)]
            assert e["T"] < 1e-2, (tau, line, e)
            assert e["ux"] < 1e-2, (tau, line, e)
            for k in ("pixx", "piyy", "pixy", "t2pee"):
                if k in e:
                    assert e[k] < 5e-2, (tau, line, k, e)
