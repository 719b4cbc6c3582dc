"""Reduced modes on the GPU against the oracle: tables with frozen
chemical-potential axes (T-only, baryon-only; src/rootfinder.cpp:447-491,
src/eos_derivatives.cpp:33-260), batch inversion in both modes and both
derivative forms, and a short FP64 evolution of a zero-charge event on the
T-only table."""
import ctypes
import dataclasses

import numpy as np
import pytest

from ccake_gb300 import api, ics
import oracle_py as O
from reduced_tables import reduced_states, reduced_table

pytestmark = pytest.mark.gpu


def relerr(a, b, floor=1e-6):
    scale = np.abs(b) + floor * np.max(np.abs(b)) + 1e-300
    return float(np.max(np.abs(a - b) / scale))


@pytest.mark.parametrize("kind", ["T", "B"])
@pytest.mark.parametrize("entropy,thermo_mode", [(0, 1), (1, 0), (1, 1)])
def test_reduced_mode_batch_parity(kind, entropy, thermo_mode):
    tab = reduced_table(kind)
    rc = ics.RunConfig(eos_kind=2, thermo_mode=thermo_mode)
    g = api.GpuHydro(rc)
    g.set_eos_table(*tab)
    ot = O.OracleTable(*tab)
    x = reduced_states(kind, 1000, 5 + entropy)
    fw = g.eos_thermo(0, x)
    col = 1 if entropy else 5
    tgt = np.column_stack([fw[:, col], fw[:, 2], fw[:, 3], fw[:, 4]])
    seeds = x * 1.03 if entropy else np.tile([580 / 197.3269804, 0, 0, 0], (x.shape[0], 1))
    xo, tho, sto, _ = O.eos_invert_batch(rc, entropy, tgt, seeds=seeds, table=ot)
    xg, thg, stg, _ = g.eos_invert(entropy, tgt, seeds)
    assert np.array_equal(stg, sto)
    assert np.mean(stg == 0) > 0.99
    ok = stg == 0
    frozen = [1, 2, 3] if kind == "T" else [2, 3]
    assert np.all(xg[ok][:, frozen] == 0.0)
    assert relerr(xg[ok][:, 0], xo[ok][:, 0]) < 1e-12
    assert np.max(np.abs(xg[ok][:, 1] - xo[ok][:, 1])) < 1e-12
    for c in (4, 5, 6, 9, 10, 12, 13):   # p s rhoB e w dw/ds dw/drhoB
        assert relerr(thg[ok][:, c], tho[ok][:, c]) < 1e-11, c


def test_zero_charge_event_on_the_T_only_table():
    tab = reduced_table("T")
    p, rc = ics.hotspots_2d(n_side=40, n_hot=5, seed=11)
    p = dataclasses.replace(p, rhoB=np.zeros_like(p.rhoB), rhoQ=np.zeros_like(p.rhoQ))
    rc = dataclasses.replace(rc, eos_kind=2, thermo_mode=0)
    gpu = api.GpuHydro(rc)
    gpu.set_eos_table(*tab)
    gpu.load(p)
    ot = O.OracleTable(*tab)
    orc = O.OracleRun(p, rc, table=ot)
    gpu.initialize()
    assert orc.initialize() == 0
    gpu.step(3)
    assert orc.step(3) == 0
    assert np.array_equal(gpu.get_int("eos_id"), orc.get_int("eos_id"))
    for f in ("x", "u0", "u1", "ext_s", "T", "e", "ext_shv0"):
        floor = 1e-5 if f[0] == "u" else 1e-6
        assert relerr(gpu.get(f), orc.get(f), floor) < 1e-10, f


def test_restrict_mu_T_ratios_parity():
    # the same rows refused by the GPU inverter and the oracle
    import fallback_scales as FS
    from ccake_gb300 import eos_table
    tab = eos_table.synthetic_table(nT=40, nmu=11)
    c5, d5 = FS.reference_fallback_scales(*tab, ics.RunConfig().freeze_out_T)
    rng = np.random.default_rng(4)
    n = 2000
    x = np.column_stack([rng.uniform(0.055, 0.3, n), rng.uniform(-0.44, 0.44, n), np.zeros(n), np.zeros(n)])
    x /= eos_table.HBARC
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1, restrict_mu_T_ratios=1)
    g = api.GpuHydro(rc)
    g.set_eos_table(*tab, c5, d5)
    ot = O.OracleTable(*tab, c5, d5)
    fw = g.eos_thermo(0, x)
    tgt = np.column_stack([fw[:, 1], fw[:, 2], fw[:, 3], fw[:, 4]])
    xo, _, sto, _ = O.eos_invert_batch(rc, 1, tgt, seeds=x.copy(), table=ot)
    xg, _, stg, _ = g.eos_invert(1, tgt, x.copy())
    assert np.mean(stg == sto) > 0.995
    # no table root above the bound
    tab_rows = stg == 0
    assert np.all(np.max(np.abs(xg[tab_rows][:, 1:]), axis=1) <= 3.5 * xg[tab_rows][:, 0])
    # against the unrestricted inversion: exactly the table roots above the
    # bound leave the table, every other row keeps its status and root
    g0 = api.GpuHydro(ics.RunConfig(eos_kind=2, thermo_mode=1))
    g0.set_eos_table(*tab, c5, d5)
    xu, _, stu, _ = g0.eos_invert(1, tgt, x.copy())
    over = (stu == 0) & (np.max(np.abs(xu[:, 1:]), axis=1) > 3.5 * xu[:, 0])
    assert over.sum() > 50
    assert np.all(stg[over] != 0)
    keep = ~over
    assert np.array_equal(stg[keep], stu[keep])
    assert np.array_equal(xg[keep & (stu == 0)], xu[keep & (stu == 0)])
