"""The viscous equations of motion pinned to the reference's own data: the
semi-analytic Israel-Stewart Gubser solutions of misc/Gubser_checks/ac
(eta/s = 0.2, tau_pi = 5 eta/w, conformal EoS e = 3p with the reference's
constant), on the CPU oracle.

1. The semi-analytic solution restated in ccake_gb300.ics.GubserIS
   reproduces every reference table (tau = 1, 1.2, 1.4, 1.5, 2 fm/c along
   y = 0; 1.2, 1.5, 2 along y = x) to the tables' printed precision. The
   tau = 1.2, 1.5 and 2.0 tables sit 1.6e-4 below the tau = 1 and 1.4 ones in
   T, a constant factor of the tabulator's run; T is held to 3e-4 there.
2. The oracle, started from that solution at tau = 1 fm/c on a 141 x 141
   lattice (dx = 0.1 fm, h = 0.2 fm) with the reference's viscous-Gubser
   settings (input/config_visc_gubser.yaml: delta_pipi "default", tau_pipi,
   lambda_piPi, phi6, phi7 "disabled"), matches the tau = 1.2 fm/c tables
   along both lines to the SPH resolution: T to 1 %, u to 1.2 % and pi to
   5 % of their largest magnitude (halving h halves these; the GPU tests
   show the convergence).
3. The same run with every second-order coefficient at its *_DEFAULT value
   (tau_pipi = 10/7 tau_pi, phi7 = 9/(70 p), ...) misses the tables by more:
   the settings matter and are honoured.
"""
import dataclasses

import numpy as np
import pytest

import gubser_tables as GT
import oracle_py as O
from ccake_gb300 import ics

HB = GT.HBARC_GEVFM


def test_solution_reproduces_reference_tables():
    sol = ics.GubserIS()
    tabs = GT.load()
    assert len(tabs) == 8
    for (line, tau), a in tabs.items():
        f = sol.fields(tau, a[:, 0], a[:, 1])
        tol_T = 1e-5 if tau in (1.0, 1.4) else 3e-4
        assert np.max(np.abs(f["T"] * HB / a[:, 2] - 1.0)) < tol_T, (line, tau)
        assert np.max(np.abs(f["ux"] - a[:, 3])) < 2e-6, (line, tau)
        assert np.max(np.abs(f["uy"] - a[:, 4])) < 2e-6, (line, tau)
        for col, k in ((5, "pixx"), (6, "piyy"), (7, "pixy"), (8, "t2pietaeta")):
            assert np.max(np.abs(f[k] * HB - a[:, col])) < 6e-5, (line, tau, k)


def _evolve(rc_changes=None, tau=1.2):
    p, rc, pi = ics.gubser_viscous_2d(n_side=141, dx=0.1, h=0.2)
    if rc_changes:
        rc = dataclasses.replace(rc, **rc_changes)
    orc = O.OracleRun(p, rc)
    orc.set_initial_viscous(None, pi)
    assert orc.initialize() == 0
    # the initial state is the solution itself (pi^{eta eta} from the constraints)
    assert np.max(np.abs(orc.get("shv33") - pi[5])) < 1e-12 * np.max(np.abs(pi[5]))
    assert orc.step(int(round((tau - rc.t0) / rc.dt))) == 0
    assert abs(orc.t - tau) < 1e-12
    fields = GT.sph_fields(orc.get, orc.t)
    return orc.get("x"), orc.get("y"), fields


def _errors(x, y, fields, tabs, tau):
    out = {}
    for line, xlim in (("y=0", 4.5), ("y=x", 3.5)):
        out[line] = GT.line_errors(tabs[(line, tau)], line, x, y, fields, 0.1, xlim)
    return out


@pytest.fixture(scope="module")
def tables():
    return GT.load()


def test_oracle_viscous_gubser_matches_reference_tables(tables):
    x, y, f = _evolve()
    err = _errors(x, y, f, tables, 1.2)
    for line, e in err.items():
        assert e["T"] < 1e-2, (line, e)
        assert e["ux"] < 1.2e-2, (line, e)
        for k in ("pixx", "piyy", "pixy", "t2pee"):
            if k in e:
                assert e[k] < 5e-2, (line, k, e)


def test_second_order_settings_are_honoured(tables):
    # all *_DEFAULT coefficients (the zeroed config) instead of the
    # Israel-Stewart settings of the reference's Gubser run
    x, y, f = _evolve(dict(tau_pipi_mode=0, lambda_piPi_mode=0, phi6_mode=0, phi7_mode=0))
    err = _errors(x, y, f, tables, 1.2)
    worst = max(err["y=0"]["piyy"], err["y=x"]["pixy"])
    assert worst > 5e-2, err
