"""The oracle's reduced modes for tables with frozen chemical-potential
axes (src/rootfinder.cpp:447-491: T-only and baryon-only root finding with
mu = 0 equations for the frozen potentials; src/eos_derivatives.cpp:33-260:
the reduced Schur complements). Without them a 4-D Newton on such a table
meets a singular Jacobian and the rows fall down the EoS chain."""
import ctypes

import numpy as np
import pytest

from ccake_gb300 import ics
import oracle_py as O
from reduced_tables import reduced_states, reduced_table


def table_thermo(cfg, ot, x):
    out = np.zeros((x.shape[0], 17))
    for i in range(x.shape[0]):
        o = np.zeros(17)
        O.lib().orc_eos_full_thermo(ctypes.byref(cfg), ot.h, 0, O._dp(x[i].copy()), O._dp(o))
        out[i] = o
    return out


@pytest.mark.parametrize("kind", ["T", "B"])
@pytest.mark.parametrize("entropy", [0, 1])
def test_reduced_mode_inversion_on_the_table(kind, entropy):
    tab = reduced_table(kind)
    ot = O.OracleTable(*tab)
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    cfg = O.make_config(rc)
    x = reduced_states(kind, 300, 3 + entropy)
    fw = table_thermo(cfg, ot, x)
    col = 1 if entropy else 5
    tgt = np.column_stack([fw[:, col], fw[:, 2], fw[:, 3], fw[:, 4]])   # (e|s, B, S, Q)
    seeds = np.tile([580 / 197.3269804, 0, 0, 0], (x.shape[0], 1))
    xo, tho, sto, _ = O.eos_invert_batch(rc, entropy, tgt, seeds=seeds, table=ot)
    assert np.mean(sto == 0) > 0.99                 # the table solves them
    ok = sto == 0
    # the frozen potentials stay at their node, zero
    frozen = [1, 2, 3] if kind == "T" else [2, 3]
    assert np.all(xo[ok][:, frozen] == 0.0)
    back = table_thermo(cfg, ot, xo[ok])
    got = np.column_stack([back[:, col], back[:, 2]])
    want = tgt[ok][:, :2]
    assert np.max(np.abs(got - want) / (np.abs(want).max(axis=0) + 1e-300)) < 1e-9
    # on a grid line the table's interpolant is exact in the frozen axes: the
    # root is the drawn state to the interpolation error of the free ones
    assert np.max(np.abs(xo[ok][:, 0] - x[ok][:, 0]) / x[ok][:, 0]) < 1e-2


@pytest.mark.parametrize("kind", ["T", "B"])
def test_reduced_mode_derivatives(kind):
    # thermo_mode 0 (the reference's Schur chain): in the reduced modes the
    # complements run over the active rows only (T-only: dw/ds = T + s/chi_TT;
    # baryon-only: the 2x2 forms of src/eos_derivatives.cpp with their 1e-30
    # guards), not over the table's stored susceptibilities of the frozen axes
    tab = reduced_table(kind)
    ot = O.OracleTable(*tab)
    rc = ics.RunConfig(eos_kind=2, thermo_mode=0)
    cfg = O.make_config(rc)
    x = reduced_states(kind, 200, 11)
    fw = table_thermo(cfg, ot, x)
    tgt = np.column_stack([fw[:, 1], fw[:, 2], fw[:, 3], fw[:, 4]])
    xo, th, st, _ = O.eos_invert_batch(rc, 1, tgt, seeds=x.copy(), table=ot)
    ok = st == 0
    assert np.mean(ok) > 0.99
    o = table_thermo(cfg, ot, xo[ok])
    T, mB, s, B = xo[ok][:, 0], xo[ok][:, 1], o[:, 1], o[:, 2]
    t2, tb, b2 = o[:, 16], o[:, 13], o[:, 7]
    if kind == "T":
        want_s = T + s / t2
        want_b = mB
    else:
        hB = np.abs(B) > 1e-25
        term1 = t2 - (tb * tb) / (b2 + 1e-30)
        term2 = tb - (t2 * b2) / (tb + 1e-30)
        term3 = tb - (b2 * t2) / (tb + 1e-30)
        term4 = b2 - (tb * tb) / (t2 + 1e-30)
        want_s = T + s / term1 + np.where(hB, B / term2, 0.0)
        want_b = mB + np.where(hB, s / term3 + B / term4, 0.0)
    assert np.allclose(th[ok][:, 12], want_s, rtol=1e-12, atol=0)
    assert np.allclose(th[ok][:, 13], want_b, rtol=1e-12, atol=1e-14)


def test_restrict_mu_T_ratios_refuses_table_roots():
    # src/eos.cpp:781-786: with restrict_mu_T_ratios a table root with
    # max |mu| > 3.5 T goes down the chain; without it the table keeps it
    import fallback_scales as FS
    from ccake_gb300 import eos_table
    tab = eos_table.synthetic_table(nT=40, nmu=11)
    c5, d5 = FS.reference_fallback_scales(*tab, ics.RunConfig().freeze_out_T)
    ot = O.OracleTable(*tab, c5, d5)
    # (T, muB) in GeV: muB / T = 3.75, 6.7 (refused); 3.0, 1.33 (kept)
    x = np.array([[0.08, 0.3, 0, 0], [0.06, 0.4, 0, 0], [0.1, 0.3, 0, 0], [0.3, 0.4, 0, 0]]) / eos_table.HBARC
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    fw = table_thermo(O.make_config(rc), ot, x)
    tgt = np.column_stack([fw[:, 1], fw[:, 2], fw[:, 3], fw[:, 4]])
    _, _, st0, _ = O.eos_invert_batch(rc, 1, tgt, seeds=x.copy(), table=ot)
    rr = ics.RunConfig(eos_kind=2, thermo_mode=1, restrict_mu_T_ratios=1)
    _, _, st1, _ = O.eos_invert_batch(rr, 1, tgt, seeds=x.copy(), table=ot)
    assert list(st0) == [0, 0, 0, 0]
    assert st1[0] > 0 and st1[1] > 0 and st1[2] == 0 and st1[3] == 0
