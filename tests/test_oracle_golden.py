"""Pins the CPU oracle against the reference's own unit-test golden values
(fixtures generated from the reference test sources by tests/golden/make_golden.py)."""
import json
import math
import os

import numpy as np
import pytest

import oracle_py as O
from ccake_gb300 import ics

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_kernel_golden_values():
    d = json.load(open(os.path.join(GOLD, "kernel_golden.json")))
    assert len(d["cases"]) >= 20
    for c in d["cases"]:
        if c["kind"] == "W":
            got = O.kernel_W(c["D"], c["r"], c["h"])
            assert abs(got - c["expect"]) < d["tol"], c
        else:
            rel = np.array(c["rel"])
            g = O.kernel_gradW(c["D"], rel, float(np.sqrt(rel @ rel)), c["h"])
            assert np.all(np.abs(g - np.array(c["expect"])) < d["tol"]), (c, g)


def _particles(pos, n_extra=0):
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    z = np.zeros(n)
    return ics.Particles(pos[:, 0].copy(), pos[:, 1].copy(), z.copy(), z + 1.0, z.copy(), z.copy(), z.copy(),
                         z.copy(), z.copy(), z.copy())


def test_smoothing_golden():
    g = json.load(open(os.path.join(GOLD, "sph_sums_golden.json")))["smoothing"]
    p = _particles(g["positions"])
    rc = ics.RunConfig(dim=2, hT=g["h"], t0=1.0)
    r = O.OracleRun(p, rc)
    n = p.n
    for k in ("s", "B", "S", "Q"):
        r.set("mass_" + k, np.ones(n))
        r.set("ext_" + k, np.ones(n))
    r.set("mass_B", 2 * np.ones(n))
    r.set("ext_B", 2 * np.ones(n))
    r.phase("neighbours")
    r.phase("velocity")
    r.phase("smooth_fields")
    assert abs(r.get("sigma_lab")[0] - g["sigma_lab_0"]) < 1e-14
    assert abs(r.get("smoothed_s")[0] - g["sigma_lab_0"]) < 1e-14
    # rho_B* with sph mass 2 and extensive 2 is four times sigma*
    assert abs(r.get("smoothed_B")[0] - 4 * g["sigma_lab_0"]) < 1e-13


def test_gradient_golden():
    g = json.load(open(os.path.join(GOLD, "sph_sums_golden.json")))["gradient"]
    p = _particles(g["positions"])
    rc = ics.RunConfig(dim=2, hT=g["h"], t0=1.0)
    r = O.OracleRun(p, rc)
    n = p.n
    r.set("mass_s", np.ones(n))
    r.set("sigma_lab", np.ones(n))
    r.set("p", np.array(g["p"]))
    r.phase("neighbours")
    r.phase("velocity")
    r.phase("gradients")
    assert abs(r.get("gradP0")[0] - g["gradP_0"][0]) < 1e-14
    assert abs(r.get("gradP1")[0] - g["gradP_0"][1]) < 1e-14


def test_isolated_particle_rk2_is_static():
    p = _particles([[0.0, 0.0]])
    p.e[:] = 10.0
    rc = ics.RunConfig(dim=2, hT=0.1, t0=1.0, dt=0.01)
    r = O.OracleRun(p, rc)
    assert r.initialize() == 0
    s0 = r.get("ext_s").copy()
    r.step(3)
    assert abs(r.t - 1.03) < 1e-14
    assert r.get("ext_s")[0] == s0[0]
    assert r.get("x")[0] == 0.0 and r.get("u0")[0] == 0.0


def _linear_table(n=(4, 3, 3, 5)):
    lo = np.array([0.5, -0.4, -0.3, -0.2])
    d = np.array([0.1, 0.2, 0.15, 0.1])
    coef = np.arange(17 * 5, dtype=np.float64).reshape(17, 5) * 0.01 + 0.1
    grids = [lo[k] + d[k] * np.arange(n[k]) for k in range(4)]
    G = np.stack(np.meshgrid(*grids, indexing="ij"), axis=-1).reshape(-1, 4)
    F = coef[:, 0][None, :] + G @ coef[:, 1:].T
    return n, lo, d, F, coef


def test_multilinear_table_is_exact_on_linear_fields():
    # unit_tests/eos_interpolator_test.cpp:44-135: a linear function is reproduced exactly
    n, lo, d, F, coef = _linear_table()
    tab = O.OracleTable(n, lo, d, F.ravel(), [1, 1, 1, 1, 1], [1, 1, 1, 1, 1])
    rc = ics.RunConfig(eos_kind=2)
    cfg = O.make_config(rc)
    rng = np.random.default_rng(0)
    hi = lo + d * (np.array(n) - 1)
    import ctypes
    for _ in range(50):
        x = lo + rng.random(4) * (hi - lo)
        out = np.zeros(17)
        O.lib().orc_eos_full_thermo(ctypes.byref(cfg), tab.h, 0, O._dp(x), O._dp(out))
        expect = coef[:, 0] + coef[:, 1:] @ x
        assert np.allclose(out, expect, rtol=0, atol=1e-12)


@pytest.mark.parametrize("eos_kind,entropy", [(0, 1), (0, 0), (1, 1), (1, 0)])
def test_eos_inversion_round_trip(eos_kind, entropy):
    rng = np.random.default_rng(7)
    n = 400
    T = rng.uniform(0.3, 2.5, n)
    mu = rng.uniform(-0.4, 0.4, (n, 3)) * (eos_kind == 1 or 1)
    rc = ics.RunConfig(eos_kind=eos_kind)
    cfg = O.make_config(rc)
    import ctypes
    tgt = np.zeros((n, 4))
    for i in range(n):
        x = np.array([T[i], mu[i, 0], mu[i, 1], mu[i, 2]])  # (T, muB, muQ, muS)
        o = np.zeros(17)
        O.lib().orc_eos_full_thermo(ctypes.byref(cfg), None, 0, O._dp(x), O._dp(o))
        tgt[i] = [o[1] if entropy else o[5], o[2], o[3], o[4]]  # (e|s, B, S, Q)
    x, th, st, it = O.eos_invert_batch(rc, entropy, tgt, seeds=np.tile([580 / 197.3269804, 0, 0, 0], (n, 1)))
    assert np.all(st >= 0)
    assert np.allclose(x[:, 0], T, rtol=1e-10, atol=0)
    assert np.allclose(x[:, 1:], mu, rtol=1e-9, atol=1e-12)


def test_reference_thermo_chain_vs_exact():
    # the reference's Schur chain (thermo_mode 0) is reproduced; it agrees with the exact
    # Hessian inverse where the reference is well defined (one charge) and returns
    # the reference's ~1e20 dw/drho when two charges are non-zero with the diagonal EoS
    import ctypes
    base = ics.RunConfig(eos_kind=1)
    T, muB, muQ = 1.5, 0.3, 0.12
    for mq, finite in ((0.0, True), (muQ, False)):
        x = np.array([T, muB, mq, 0.0])
        res = {}
        for mode in (0, 1):
            rc = ics.RunConfig(eos_kind=1, thermo_mode=mode)
            th = np.zeros(16)
            O.lib().orc_eos_set_thermo(ctypes.byref(O.make_config(rc)), None, 0, O._dp(x), O._dp(th))
            res[mode] = th
        assert abs(res[1][12] - 4 * T / 3) < 1e-12
        assert abs(res[1][13] - 4 * muB / 3) < 1e-12
        if finite:
            assert abs(res[0][12] - res[1][12]) < 1e-10 * T
            assert abs(res[0][13] - res[1][13]) < 1e-10 * muB
        else:
            assert abs(res[0][13]) > 1e15


def test_gubser_against_analytic():
    p, rc = ics.gubser_2d(n_side=80)
    r = O.OracleRun(p, rc)
    assert r.initialize() == 0
    tot0 = r.totals()
    assert r.step(20) == 0
    x, y, T = r.get("x"), r.get("y"), r.get("T")
    rr = np.sqrt(x * x + y * y)
    m = rr < 1.5
    Ta = ics.gubser_temperature(r.t, rr)
    assert np.max(np.abs(T[m] / Ta[m] - 1)) < 5e-3
    tot = r.totals()
    assert abs(tot["S"] / tot0["S"] - 1) < 1e-12          # ideal: entropy conserved
    assert abs((tot["E"] + tot["Ez"]) / tot0["E"] - 1) < 2e-3


def test_table_jacobian_is_the_interpolant_derivative():
    # the Newton Jacobian of the table model: derivatives of the multilinear
    # interpolant of s, rho and e, against central differences inside a cell
    import ctypes
    from ccake_gb300 import eos_table
    n, lo, d, f = eos_table.synthetic_table(nT=9, nmu=5)
    c5, d5 = eos_table.fallback_scales()
    t = O.OracleTable(n, lo, d, f, c5, d5)
    L = O.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    L.orc_table_jacobian.argtypes = [ctypes.c_void_p, dp, dp, dp]
    rng = np.random.default_rng(5)
    for _ in range(20):
        cell = rng.integers(0, n - 1)
        frac = rng.uniform(0.2, 0.8, 4)
        x = lo + d * (cell + frac)
        o, jac = np.zeros(17), np.zeros(20)
        L.orc_table_jacobian(t.h, O._dp(x), O._dp(o), O._dp(jac))
        jac = jac.reshape(5, 4)
        for j in range(4):
            h = 1e-4 * d[j]
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            op, om = np.zeros(17), np.zeros(17)
            L.orc_table_jacobian(t.h, O._dp(xp), O._dp(op), O._dp(np.zeros(20)))
            L.orc_table_jacobian(t.h, O._dp(xm), O._dp(om), O._dp(np.zeros(20)))
            fd = (op[1:6] - om[1:6]) / (2 * h)
            assert np.allclose(jac[:, j], fd, rtol=1e-6, atol=1e-9 * np.abs(fd).max()), j
