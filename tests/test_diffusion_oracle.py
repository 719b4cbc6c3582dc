"""The oracle's diffusion sector on the CPU: the alpha derivatives against
finite differences of the EoS inversion, the reference's derivative chain
against the exact Hessian inverse where the chain is regular, the regulator
cap, and an event that moves charge while keeping it."""
import dataclasses

import numpy as np

from ccake_gb300 import ics
import oracle_py as O


def _alpha(rc, tgt, seed):
    x, th, st, _ = O.eos_invert_batch(rc, 1, tgt[None, :], seeds=seed)
    assert st[0] == 0
    return np.array([th[0, 1], th[0, 2], th[0, 3]]) / th[0, 0], x   # muB, muS, muQ over T


def test_alpha_derivatives_match_finite_differences():
    # conformal-diagonal EoS, all three charges non-zero, exact inverse
    rc = ics.RunConfig(eos_kind=1, thermo_mode=1)
    tgt = np.array([20.0, 0.5, 0.1, 0.2])
    a0, x = _alpha(rc, tgt, np.array([[1.0, 0.1, 0.1, 0.1]]))
    da = O.eos_alpha_derivs(rc, 0, x)[0]
    fd = np.zeros(12)
    for j in range(4):
        h = 1e-6 * max(abs(tgt[j]), 1.0)
        tp, tm = tgt.copy(), tgt.copy()
        tp[j] += h
        tm[j] -= h
        d = (_alpha(rc, tp, x)[0] - _alpha(rc, tm, x)[0]) / (2 * h)
        if j == 0:
            fd[0:3] = d
        else:
            for a in range(3):
                fd[3 + 3 * a + (j - 1)] = d[a]
    assert np.allclose(da, fd, rtol=1e-6, atol=1e-10 * np.max(np.abs(fd)))


def test_alpha_chain_matches_exact_inverse_where_regular():
    # conformal EoS: the Schur-complement chain of src/eos.cpp equals H^-1
    for charges in ((0.5, 0.1, 0.2), (0.5, 0.0, 0.0)):
        out = []
        for tm in (0, 1):
            rc = ics.RunConfig(eos_kind=0, thermo_mode=tm)
            x, _, st, _ = O.eos_invert_batch(rc, 1, np.array([[20.0, *charges]]),
                                             seeds=np.array([[1.0, 0.1, 0.1, 0.1]]))
            assert st[0] == 0
            out.append(O.eos_alpha_derivs(rc, 0, x)[0])
        scale = np.max(np.abs(out[1]))
        assert np.allclose(out[0], out[1], rtol=1e-12, atol=1e-14 * scale), charges
    # baryon only: the S and Q rows vanish
    assert np.all(np.abs(out[0][[4, 5, 6, 7, 8, 9, 10, 11]]) < 1e-100)


def test_regulator_caps_the_current():
    p, rc = ics.hotspots_2d(n_side=24, n_hot=3, seed=13)
    # e above the regulator's e0 = 0.1 GeV/fm^3 everywhere, so that its
    # strength is near chi0 and part of the current stays below the cap
    p = dataclasses.replace(p, e=50.0 * p.e, rhoB=10.0 * p.rhoB, rhoQ=np.zeros_like(p.rhoQ))
    rc = dataclasses.replace(rc, eos_kind=0, thermo_mode=0, using_diffusion=1, diffusion_mode=2,
                             diffusion_relax_mode=1, C_B=0.4, diffusion_regulator=1)
    o = O.OracleRun(p, rc)
    o.set("in_qB1", 15.0 * p.rhoB * np.cos(6.0 * p.x))
    assert o.initialize() == 0
    for ph in ("neighbours", "velocity", "smooth_fields", "thermo", "reset_pi"):
        o.phase(ph)
    n = np.abs(o.get("rhoB"))
    before = np.sqrt(np.maximum(o.get("qB1") ** 2 + o.get("qB2") ** 2 - o.get("qB0") ** 2, 0)) / n
    o.phase("regulate_diffusion")
    after = np.sqrt(np.maximum(o.get("qB1") ** 2 + o.get("qB2") ** 2 - o.get("qB0") ** 2, 0)) / n
    # f(e) = chi0 (Fermi(e) - Fermi(0)) ~ 10 for e >> e0 = 0.1 GeV/fm^3
    assert before.max() > 12.0
    assert after.max() <= 10.0 * (1 + 1e-12)
    capped = after < before * (1 - 1e-12)
    assert capped.any() and (~capped).any()
    assert np.allclose(after[~capped], before[~capped], rtol=1e-14)


def test_diffusion_moves_charge_and_keeps_it():
    p, rc = ics.hotspots_2d(n_side=24, n_hot=3, seed=11)
    rc = dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=(0.3, 0, 0, 0, 0, 0, 0, 0, 0.3))
    o = O.OracleRun(p, rc)
    assert o.initialize() == 0
    b0, t0 = o.get("ext_B"), o.totals()
    assert o.step(10) == 0
    t1 = o.totals()
    moved = np.max(np.abs(o.get("ext_B") - b0))
    assert moved > 1e-6 * np.max(np.abs(b0))
    # net baryon charge (with the q^0 terms) changes far less than it moves
    assert abs(t1["B"] - t0["B"]) < 0.1 * moved * p.n
    assert abs(t1["B"] - t0["B"]) < 1e-4 * abs(t0["B"])
    assert np.isfinite(o.get("u0")).all() and np.max(np.abs(o.get("qB1"))) > 0


def test_diffusion_coefficients_follow_their_modes():
    # constant_over_T2: kappa = kappa/T^2 T^2, tau_q = 0.2/T on the diagonal;
    # kappaB_coth: kappa_B = (C_B/T) n_B ((1/3) coth(mu_B/T) - n_B T/w) where
    # |mu_B/T| > 1e-2 and the value is positive, tau_q = C_B/T
    # (src/transport_coefficients.cpp:918-1040)
    p, rc = ics.hotspots_2d(n_side=20, n_hot=2, seed=13)
    kap = (0.3, 0.01, 0.0, 0.01, 0.2, 0.0, 0.0, 0.0, 0.1)
    o = O.OracleRun(p, dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=kap))
    assert o.initialize() == 0 and o.step(1) == 0
    T = o.get("T")
    for c, C in enumerate("BSQ"):
        for d, Dd in enumerate("BSQ"):
            assert np.allclose(o.get(f"kappa_q{C}{Dd}"), kap[3 * c + d] * T * T, rtol=1e-15, atol=0)
            assert np.allclose(o.get(f"tau_q{C}{Dd}"), (0.2 / T) if c == d else 0.0, rtol=1e-15, atol=0)
    # a baryon profile whose mu_B/T straddles the 1e-2 floor
    p2 = dataclasses.replace(p, e=50.0 * p.e, rhoB=400.0 * p.rhoB * (0.5 + 0.5 * np.cos(6.0 * p.x)),
                             rhoQ=np.zeros_like(p.rhoQ))
    rc2 = dataclasses.replace(rc, eos_kind=0, thermo_mode=0, using_diffusion=1, diffusion_mode=2,
                              diffusion_relax_mode=1, C_B=0.4)
    o2 = O.OracleRun(p2, rc2)
    assert o2.initialize() == 0 and o2.step(1) == 0
    T, muB, nB, w = o2.get("T"), o2.get("muB"), o2.get("rhoB"), o2.get("w")
    x = muB / T
    kB = (0.4 / T) * nB * ((1.0 / 3.0) / np.tanh(x) - nB * T / w)
    want = np.where((np.abs(x) > 1e-2) & (kB > 0), kB, 0.0)
    assert np.any(want > 0) and np.any(want == 0)
    assert np.allclose(o2.get("kappa_qBB"), want, rtol=1e-13, atol=0)
    assert np.all(o2.get("kappa_qSS") == 0) and np.all(o2.get("kappa_qBQ") == 0)
    assert np.allclose(o2.get("tau_qBB"), 0.4 / T, rtol=1e-15) and np.allclose(o2.get("tau_qQQ"), 0.4 / T, rtol=1e-15)


def test_cartesian_diffusion_runs_and_keeps_charge():
    p, rc = ics.hotspots_2d(n_side=24, n_hot=3, seed=11)
    rc = dataclasses.replace(rc, coord=1, using_diffusion=1, kappa_over_T2=(0.3, 0, 0, 0, 0, 0, 0, 0, 0.3))
    o = O.OracleRun(p, rc)
    assert o.initialize() == 0
    b0, t0 = o.get("ext_B"), o.totals()
    assert o.step(10) == 0
    assert np.max(np.abs(o.get("ext_B") - b0)) > 1e-6 * np.max(np.abs(b0))
    assert abs(o.totals()["B"] - t0["B"]) < 1e-4 * abs(t0["B"])


def test_critical_point_suppression_with_the_table_eos():
    # default_kappa with critical_scaling: kappa = (1 - exp(-[(T - T_c)^2 /
    # (2 w_T^2) + (mu_B - mu_Bc)^2 / (2 w_mu^2)])) kappa/T^2 T^2 where the
    # particle's EoS is the table (src/transport_coefficients.cpp:942-948,
    # :1048-1057); inputs in MeV, converted to fm^-1
    from ccake_gb300 import eos_table
    n, lo, d, f = eos_table.synthetic_table(nT=76, nmu=21)
    ot = O.OracleTable(n, lo, d, f, *eos_table.fallback_scales())
    p, rc = ics.hotspots_2d(n_side=16, n_hot=3, seed=11, floor_GeV=4.0, peak_range=(5.0, 30.0))
    rc = dataclasses.replace(rc, eos_kind=2, using_diffusion=1, kappa_over_T2=(0.3, 0, 0, 0, 0, 0, 0, 0, 0.3),
                             critical_scaling_diffusion=1, crit_T=300.0, crit_muB=100.0, crit_wT=60.0,
                             crit_wmuB=200.0)
    o = O.OracleRun(p, rc, table=ot)
    assert o.initialize() == 0 and o.step(1) == 0
    hc = 197.3269804
    T, muB = o.get("T"), o.get("muB")
    ex = 0.5 * ((T - 300.0 / hc) ** 2 / (60.0 / hc) ** 2 + (muB - 100.0 / hc) ** 2 / (200.0 / hc) ** 2)
    table = o.get_int("eos_id") == 0
    sup = np.where(table, 1.0 - np.exp(-ex), 1.0)
    assert table.any()
    assert np.allclose(o.get("kappa_qBB"), sup * 0.3 * T * T, rtol=1e-12, atol=0)
    assert np.min(sup[table]) < 0.999
