"""The tanh-conformal fallback of the table EoS chain in the oracle
(include/eos_tanh_conformal.h; chain table -> tanh_conformal -> conformal ->
conformal_diagonal, src/eos_initialization.cpp:270-464 with
use_tanh_conformal = true, include/eos_header.h:7).

* Its densities and susceptibilities are the derivatives of its pressure
  (finite differences), and its c_s^2 is dp/de along fixed s : rho ratios.
* In the table chain it sits at index 1: a state the table cannot hold
  (T above the grid) is solved by it, in both inversion modes.
* The fallback scales follow the reference's matching to the table.
"""
import ctypes

import numpy as np
import pytest

import fallback_scales as FS
import oracle_py as O
from ccake_gb300 import eos_table, ics

TANH = 1


@pytest.fixture(scope="module")
def table():
    n, lo, d, f = eos_table.synthetic_table(nT=31, nmu=9)
    conf5, cdiag5 = FS.reference_fallback_scales(n, lo, d, f, 150.0 / 197.3269804)
    return n, lo, d, f, conf5, cdiag5


def thermo(table, k, x):
    ot = O.OracleTable(*table)
    cfg = O.make_config(ics.RunConfig(eos_kind=2, thermo_mode=1))
    out = np.zeros(17)
    O.lib().orc_eos_full_thermo(ctypes.byref(cfg), ot.h, k, O._dp(np.asarray(x, dtype=np.float64)), O._dp(out))
    return out


def test_fallback_scales_follow_the_reference_matching(table):
    n, lo, d, f, conf5, cdiag5 = table
    Tmax = 1.1 * 150.0 / 197.3269804
    p = lambda x: thermo(table, 0, x)[0]
    c = p([Tmax, 0, 0, 0]) / Tmax ** 4
    assert conf5[0] == pytest.approx(c, rel=1e-14) and conf5[1] == 1.0
    muBmax = lo[1] + d[1] * (n[1] - 1)
    pB = p([Tmax, muBmax, 0, 0])
    assert conf5[2] == pytest.approx(c ** 0.25 * muBmax / np.sqrt(np.sqrt(pB) - np.sqrt(p([Tmax, 0, 0, 0]))),
                                     rel=1e-14)
    assert cdiag5[2] == pytest.approx((c / (pB - p([Tmax, 0, 0, 0]))) ** 0.25 * muBmax, rel=1e-14)
    # the conformal fallback (chain index 2) of this matching meets the
    # table's pressure at (Tmax, muB_max, 0, 0)
    assert thermo(table, 2, [Tmax, muBmax, 0, 0])[0] == pytest.approx(pB, rel=1e-12)


@pytest.mark.parametrize("x", [[1.2, 0.3, -0.1, 0.2], [0.6, -0.5, 0.2, 0.0], [3.0, 0.8, 0.4, -0.6],
                               [0.9, 0.0, 0.0, 0.0]])
def test_tanh_conformal_is_thermodynamically_consistent(table, x):
    x = np.array(x)
    o = thermo(table, TANH, x)
    h = 1e-5
    grad = np.zeros(4)
    hess = np.zeros((4, 4))
    dens = lambda y: np.array([thermo(table, TANH, y)[i] for i in (1, 2, 4, 3)])   # s, B, Q, S
    for j in range(4):
        e = np.zeros(4)
        e[j] = h * max(1.0, abs(x[j]))
        grad[j] = (thermo(table, TANH, x + e)[0] - thermo(table, TANH, x - e)[0]) / (2 * e[j])
        hess[:, j] = (dens(x + e) - dens(x - e)) / (2 * e[j])
    assert np.allclose(grad, [o[1], o[2], o[4], o[3]], rtol=1e-8)
    H = np.array([[o[16], o[13], o[14], o[15]], [o[13], o[7], o[10], o[11]], [o[14], o[10], o[8], o[12]],
                  [o[15], o[11], o[12], o[9]]])
    assert np.allclose(hess, H, rtol=1e-6, atol=1e-8 * np.abs(H).max())
    T, mB, mQ, mS = x
    w = o[1] * T + mB * o[2] + mQ * o[4] + mS * o[3]
    assert o[5] == pytest.approx(w - o[0], rel=1e-14)
    # c_s^2 = dp/de along dn = n dlambda (fixed s : rho), by finite steps
    n0 = np.array([o[1], o[2], o[4], o[3]])
    step = 1e-6
    xs = [x + np.linalg.solve(H, n0 * lam) for lam in (-step, step)]
    oo = [thermo(table, TANH, y) for y in xs]
    cs2 = (oo[1][0] - oo[0][0]) / (oo[1][5] - oo[0][5])
    assert o[6] == pytest.approx(cs2, rel=1e-6)
    assert 0.0 < o[6] < 1.0


def test_table_chain_falls_to_tanh_conformal_above_the_grid(table):
    n, lo, d, f, conf5, cdiag5 = table
    ot = O.OracleTable(*table)
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    Tmax = lo[0] + d[0] * (n[0] - 1)
    xs = np.array([[1.3 * Tmax, 0.2, 0.05, -0.1], [2.0 * Tmax, -0.3, 0.0, 0.1]])
    for entropy, col in ((0, 5), (1, 1)):
        tgt = np.array([[thermo(table, TANH, x)[i] for i in (col, 2, 3, 4)] for x in xs])
        seeds = np.tile([580 / 197.3269804, 0, 0, 0], (len(xs), 1))
        xo, th, st, _ = O.eos_invert_batch(rc, entropy, tgt, seeds=seeds, table=ot)
        assert list(st) == [TANH, TANH]
        assert np.allclose(xo, xs, rtol=1e-9, atol=1e-9)
