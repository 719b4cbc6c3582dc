"""Mixed-precision form (precision = 1) against the FP64 oracle, through the C ABI.

The mixed form runs the pair loops in FP32 with compensated sums and the
equations of motion in FP32; the EoS, the state and the RK2 update stay FP64.
Bar: after 100 RK2 steps the local densities (e, rho_B, s, T) agree with the
FP64 oracle to 1e-5 relative per particle, the flow velocity to 1e-5 of its
range, the totals to 1e-6.
"""
import numpy as np
import pytest

from ccake_gb300 import api, ics
import oracle_py as O

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-5


def relerr(a, b, floor=1e-6):
    scale = np.abs(b) + floor * np.max(np.abs(b)) + 1e-300
    return float(np.max(np.abs(a - b) / scale))


def mixed_run(p, rc):
    rc = ics.RunConfig(**{**rc.__dict__, "precision": 1})
    g = api.GpuHydro(rc)
    g.load(p)
    g.initialize()
    return g


def test_mixed_hundred_steps_against_fp64_oracle():
    p, rc = ics.hotspots_2d(n_side=100, n_hot=10, seed=5)
    g = mixed_run(p, rc)
    orc = O.OracleRun(p, rc)
    assert orc.initialize() == 0
    g.step(100)
    assert orc.step(100) == 0
    assert abs(g.t - orc.t) < 1e-12
    for f in ("e", "rhoB", "rhoQ", "s", "T", "p", "sigma_lab", "ext_s"):
        assert relerr(g.get(f), orc.get(f)) < MIXED_RTOL, f
    for f in ("x", "y"):   # positions against the box size (they cross zero)
        assert relerr(g.get(f), orc.get(f), floor=1.0) < 1e-9, f
    for f in ("u0", "u1", "shv11", "shv12", "ext_shv0"):
        assert relerr(g.get(f), orc.get(f), floor=1e-2) < MIXED_RTOL, f
    tg, to = g.totals(), orc.totals()
    for k in ("S", "B", "Q", "E"):
        assert abs(tg[k] - to[k]) <= 1e-6 * abs(to[k]), k
    # the neighbour counts differ from the FP64 ones only by pairs at 2h
    assert np.max(np.abs(g.get_int("btrack") - orc.get_int("btrack"))) <= 4


def test_mixed_three_d_against_fp64_oracle():
    p, rc = ics.hotspots_3d(n_xy=16, n_eta=12, n_hot=4, seed=3)
    g = mixed_run(p, rc)
    orc = O.OracleRun(p, rc)
    assert orc.initialize() == 0
    g.step(10)
    assert orc.step(10) == 0
    for f in ("e", "rhoB", "s", "T", "sigma_lab"):
        assert relerr(g.get(f), orc.get(f)) < MIXED_RTOL, f
    for f in ("u0", "u1", "u2", "shv33", "ext_shv4"):
        assert relerr(g.get(f), orc.get(f), floor=1e-2) < MIXED_RTOL, f


def test_mixed_runs_are_bitwise_reproducible():
    p, rc = ics.hotspots_2d(n_side=48, n_hot=6, seed=7)
    outs = []
    for _ in range(2):
        g = mixed_run(p, rc)
        g.step(5)
        outs.append(np.concatenate([g.get("u0"), g.get("ext_shv0"), g.get("T")]))
    assert np.array_equal(outs[0], outs[1])


def test_phase_calls_between_mixed_steps_leave_the_run_unchanged():
    # the phase entry points run the FP64 form; the mixed records are
    # re-packed from the state before the next mixed step (the FP64 EoS call
    # moves the next Newton seed, hence agreement to the Newton tolerance)
    p, rc = ics.hotspots_2d(n_side=48, n_hot=6, seed=7)
    a = mixed_run(p, rc)
    a.step(6)
    b = mixed_run(p, rc)
    b.step(3)
    b.phase("smooth_fields")
    b.phase("update_thermo")
    b.step(3)
    for f in ("x", "u0", "ext_s", "ext_shv0", "T"):
        assert relerr(b.get(f), a.get(f), floor=1e-3) < 1e-9, f
