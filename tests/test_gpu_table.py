"""Tabulated EoS (eos_kind 2) on the GPU against the oracle, through the C ABI.

Table: the synthetic stress-test EoS of ccake_gb300.eos_table at reduced
resolution (76 x 21^3 nodes, 95 MB), with the EoS chain of the reference:
table -> tanh_conformal -> conformal -> conformal_diagonal, the fallbacks
matched to the table at 1.1 T_FO as the reference does. Strict parity is
checked where that EoS is thermodynamically stable (T >= 0.2 GeV:
positive-definite Hessian, so the inverse is unique); in the unstable band
T ~ 0.10-0.19 GeV the c_s^2 guard sends rows down the chain, and the rows
that land on the tanh-conformal stage are compared there.
"""
import ctypes

import numpy as np
import pytest

import fallback_scales as FS
from ccake_gb300 import api, eos_table, ics
import oracle_py as O

pytestmark = pytest.mark.gpu

NT, NMU = 76, 21
TANH = 1


def relerr(a, b, floor=1e-6):
    scale = np.abs(b) + floor * np.max(np.abs(b)) + 1e-300
    return float(np.nanmax(np.abs(a - b) / scale))


@pytest.fixture(scope="module")
def table():
    n, lo, d, f = eos_table.synthetic_table(nT=NT, nmu=NMU)
    conf5, cdiag5 = FS.reference_fallback_scales(n, lo, d, f, ics.RunConfig().freeze_out_T)
    return n, lo, d, f, conf5, cdiag5


def test_fallback_scales_match_the_reference_rule(table):
    n, lo, d, f, conf5, cdiag5 = table
    c5, d5 = api.table_fallback_scales(n, lo, d, f, ics.RunConfig().freeze_out_T)
    assert np.allclose(c5, conf5, rtol=1e-13) and np.allclose(d5, cdiag5, rtol=1e-13)
    # the context matches them itself when none are given
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    g1, g2 = api.GpuHydro(rc), api.GpuHydro(rc)
    g1.set_eos_table(n, lo, d, f)
    g2.set_eos_table(*table)
    x = np.array([[3.0, 0.2, 0.1, -0.1], [5.0, 1.0, 0.3, 0.2]])
    for k in (1, 2, 3):
        assert np.allclose(g1.eos_thermo(k, x), g2.eos_thermo(k, x), rtol=1e-12, atol=0), k


def test_tanh_conformal_thermo_parity(table):
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    g = gpu_with_table(rc, table)
    ot = O.OracleTable(*table)
    cfg = O.make_config(rc)
    rng = np.random.default_rng(17)
    x = np.column_stack([rng.uniform(0.1, 8.0, 500), rng.uniform(-2, 2, (500, 3))])
    og = g.eos_thermo(TANH, x)
    for i in range(x.shape[0]):
        o = np.zeros(17)
        O.lib().orc_eos_full_thermo(ctypes.byref(cfg), ot.h, TANH, O._dp(x[i].copy()), O._dp(o))
        assert np.allclose(og[i], o, rtol=1e-12, atol=1e-13 * np.abs(o).max()), i


def gpu_with_table(rc, table):
    g = api.GpuHydro(rc)
    g.set_eos_table(*table)
    return g


def states(n, seed, Tmin=None):
    """n states uniform in the table box; with Tmin (GeV) T uniform in [Tmin, 0.79 GeV]."""
    x = eos_table.sample_states(n, seed=seed)
    if Tmin is not None:
        x[:, 0] = np.random.default_rng(seed).uniform(Tmin, 0.79, n) / eos_table.HBARC
    return x


def test_table_lookup_parity(table):
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    g = gpu_with_table(rc, table)
    ot = O.OracleTable(*table)
    cfg = O.make_config(rc)
    x = states(3000, 1)
    n, lo, d = table[0], table[1], table[2]
    # exact nodes and the upper edges; points within one spacing outside the
    # table are extrapolated by the reference's truncating index rule
    # (src/interpolatorND.cpp:250-317), points beyond that are NaN
    x[:10] = lo + d * np.array([[0, 0, 0, 0], [1, 2, 3, 4], [NT - 1, NMU - 1, NMU - 1, NMU - 1]] * 3 + [[5, 5, 5, 5]])
    x[10:14] = lo - d * 1.5
    x[14:18] = lo + d * (n - 1) + d * 1.5
    x[18:22] = lo - d * 0.5
    og = g.eos_thermo(0, x)
    oo = np.zeros_like(og)
    for i in range(x.shape[0]):
        o = np.zeros(17)
        O.lib().orc_eos_full_thermo(ctypes.byref(cfg), ot.h, 0, O._dp(x[i].copy()), O._dp(o))
        oo[i] = o
    assert np.array_equal(np.isnan(og), np.isnan(oo))
    assert np.isnan(og[10:18]).all()
    assert not np.isnan(og[18:22]).any()
    ok = ~np.isnan(oo[:, 0])
    for c in range(17):
        assert relerr(og[ok, c], oo[ok, c], floor=1e-9) < 1e-12, c
    # nodes reproduce the generator's values
    f = table[3]
    node0 = f[0]
    assert np.allclose(og[0], node0, rtol=1e-13, atol=0)


@pytest.mark.parametrize("entropy", [0, 1])
def test_table_inversion_parity(table, entropy):
    # T >= 0.2 GeV. This EoS is not globally invertible (a state can share
    # (e|s, rho) with one in the unstable band), and from the far 580 MeV seed
    # of energy mode Newton can cross the near-singular band, where rounding
    # differences (FMA on the GPU, none in the oracle) choose between roots.
    # So: the same chain decision on >= 99.5 % of rows, both codes reproduce
    # the targets on every row they solve with the table, and the same root
    # on >= 99 % of those rows.
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    g = gpu_with_table(rc, table)
    ot = O.OracleTable(*table)
    x = states(3000, 2 + entropy, Tmin=0.2)
    fw = g.eos_thermo(0, x)
    col = 1 if entropy else 5
    tgt = np.column_stack([fw[:, col], fw[:, 2], fw[:, 3], fw[:, 4]])
    seeds = np.tile([580 / 197.3269804, 0, 0, 0], (x.shape[0], 1))
    if entropy:   # hydro-like seeds: a nearby previous state
        seeds = x * (1 + 0.05 * np.random.default_rng(9).uniform(-1, 1, x.shape))
    xo, tho, sto, _ = O.eos_invert_batch(rc, entropy, tgt, seeds=seeds, table=ot)
    xg, thg, stg, itg = g.eos_invert(entropy, tgt, seeds)
    assert np.mean(stg == sto) >= 0.995
    assert np.mean(stg == 0) > 0.99      # the table root is accepted
    both = (stg == 0) & (sto == 0)
    for xs in (xg, xo):
        r = g.eos_thermo(0, xs[both])
        back = np.column_stack([r[:, col], r[:, 2], r[:, 3], r[:, 4]])
        assert np.max(np.abs(back - tgt[both]) / (np.abs(tgt[both]).max(axis=0) + 1e-300)) < 1e-9
    same = (np.abs(xg[both, 0] / xo[both, 0] - 1) < 1e-9) & np.all(np.abs(xg[both, 1:] - xo[both, 1:]) < 1e-9, axis=1)
    assert np.mean(same) >= 0.99
    for c in (4, 5, 9, 10):
        assert relerr(thg[both][same, c], tho[both][same, c]) < 1e-9, c
    # most rows recover the drawn state itself
    rec = np.abs(xg[stg == 0, 0] / x[stg == 0, 0] - 1) < 1e-8
    assert np.mean(rec) > 0.95


def test_table_inversion_statuses_across_the_unstable_band(table):
    # states over the whole table; where the EoS is unstable the reference's
    # cs2 guard sends the solution down the chain; the GPU takes the same
    # decisions as the oracle on (nearly) every row
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    g = gpu_with_table(rc, table)
    ot = O.OracleTable(*table)
    x = states(2000, 4)
    fw = g.eos_thermo(0, x)
    tgt = np.column_stack([fw[:, 5], fw[:, 2], fw[:, 3], fw[:, 4]])
    seeds = np.tile([580 / 197.3269804, 0, 0, 0], (x.shape[0], 1))
    xo, tho, sto, _ = O.eos_invert_batch(rc, 0, tgt, seeds=seeds, table=ot)
    xg, thg, stg, _ = g.eos_invert(0, tgt, seeds)
    assert np.mean(stg == sto) > 0.995
    # rows the table rejects land on the tanh-conformal stage in both, with
    # the same roots and thermodynamics there
    tanh = (stg == TANH) & (sto == TANH)
    assert tanh.sum() >= 10 and tanh.sum() >= 0.9 * np.count_nonzero((stg == TANH) | (sto == TANH))
    assert relerr(xg[tanh, 0], xo[tanh, 0]) < 1e-10
    assert np.max(np.abs(xg[tanh, 1:] - xo[tanh, 1:])) < 1e-10
    for c in (4, 5, 9, 10, 11):
        assert relerr(thg[tanh, c], tho[tanh, c]) < 1e-10, c


def hot_table_event():
    # a 2+1-D hot-spot event that stays above the unstable band (floor
    # 4 GeV/fm^3, T > 0.2 GeV), table EoS, shear
    p, rc = ics.hotspots_2d(n_side=40, n_hot=5, seed=11, floor_GeV=4.0, peak_range=(5.0, 30.0))
    rc = ics.RunConfig(**{**rc.__dict__, "eos_kind": 2})
    return p, rc


@pytest.mark.parametrize("precision", [0, 1])
def test_table_eos_hydro_parity(table, precision):
    p, rc = hot_table_event()
    rcg = ics.RunConfig(**{**rc.__dict__, "precision": precision})
    g = gpu_with_table(rcg, table)
    g.load(p)
    g.initialize()
    ot = O.OracleTable(*table)
    orc = O.OracleRun(p, rc, table=ot)
    assert orc.initialize() == 0
    for f in ("T", "muB", "e", "s", "sigma_lab"):
        assert relerr(g.get(f), orc.get(f)) < 1e-10, f
    g.step(5)
    assert orc.step(5) == 0
    tol = 1e-10 if precision == 0 else 1e-5
    for f in ("T", "muB", "e", "ext_s"):
        assert relerr(g.get(f), orc.get(f), floor=1e-3) < tol, f
    # velocities and shear start at zero: checked against 1e-2 of their range
    for f in ("u0", "shv11"):
        assert relerr(g.get(f), orc.get(f), floor=1e-2) < tol, f
    assert np.array_equal(g.get_int("eos_id"), orc.get_int("eos_id"))


def test_three_d_table_eos_with_bulk_parity(table):
    # 3+1-D Milne lattice with the table EoS, shear and peaked bulk
    # viscosity, FP64 form against the oracle
    p, rc = ics.hotspots_3d(n_xy=14, n_eta=10, n_hot=3, seed=5, eos_kind=2, zeta_over_s=0.1, floor_GeV=4.0,
                            peak_range=(5.0, 20.0))
    g = gpu_with_table(rc, table)
    g.load(p)
    g.initialize()
    ot = O.OracleTable(*table)
    orc = O.OracleRun(p, rc, table=ot)
    assert orc.initialize() == 0
    g.step(3)
    assert orc.step(3) == 0
    for f in ("T", "muB", "e", "ext_s", "ext_bulk", "sigma_lab"):
        assert relerr(g.get(f), orc.get(f), floor=1e-3) < 1e-10, f
    for f in ("u0", "u2", "shv33", "bulk"):
        assert relerr(g.get(f), orc.get(f), floor=1e-2) < 1e-10, f


def test_learned_seed_initialisation_finds_the_same_states(table):
    # seed_mode learned: the trained seed network supplies the first seed of
    # every particle's e -> (T, mu) inversion at initialisation; where the
    # root is unique (this event stays above the unstable band) the states
    # are the reference seeds' states
    import dataclasses
    p, rc = hot_table_event()
    ref = gpu_with_table(rc, table)
    ref.load(p)
    ref.initialize()
    g = gpu_with_table(dataclasses.replace(rc, seed_mode=2), table)
    g.mlp_train(n_samples=300_000, epochs=8, batch=16384, seed=3)
    g.load(p)
    g.initialize()
    for f in ("T", "muB", "muQ", "s", "e", "sigma_lab"):
        assert relerr(g.get(f), ref.get(f)) < 1e-10, f
    assert np.array_equal(g.get_int("eos_id"), ref.get_int("eos_id"))
    # without a trained network the context refuses to initialise
    h = gpu_with_table(dataclasses.replace(rc, seed_mode=2), table)
    h.load(p)
    with pytest.raises(api.CcakeError):
        h.initialize()
