"""Failure statuses of the C ABI, each provoked by its input and turned into a
status by the library's own checks (host validation, or the kernels' error
counters with bounded loops): nothing here faults, traps or hangs the GPU.

Reference behaviour replaced (paths within the reference project):
* no EoS solution at initialisation: the particle is frozen and retried at
  zero charge, and a second failure throws (src/sph_workstation.cpp:1825-1848)
  -> CCAKE_ERR_EOS, the particle's eos_id -1;
* negative entropy after an RK update aborts unless the particle is frozen
  (src/evolver.cpp:437-450) -> CCAKE_ERR_NEG_ENTROPY;
* a failed root search returns false with the reason printed
  (src/eos.cpp:790-801) -> status -1 in the batch inversion;
* an unreadable EoS table aborts (src/eos_table.cpp:14-100) ->
  CCAKE_ERR_INVALID, the context still usable.
"""
import dataclasses

import numpy as np
import pytest

from ccake_gb300 import api, eos_table, ics
import oracle_py as O

pytestmark = pytest.mark.gpu

INVALID, EOS, NEG_ENTROPY, CAPACITY = 1, 3, 4, 5


def _expect(code, fn, *a):
    with pytest.raises(api.CcakeError) as ei:
        fn(*a)
    assert ei.value.code == code, str(ei.value)
    return str(ei.value)


def test_non_finite_energy_is_an_eos_failure_with_a_particle_status():
    p, rc = ics.hotspots_2d(n_side=24, n_hot=3, seed=2)
    bad = 100
    p.e[bad] = np.nan
    g = api.GpuHydro(rc)
    g.load(p)
    msg = _expect(EOS, g.initialize)
    assert "1 particles without an EoS solution" in msg
    eid = g.get_int("eos_id")
    assert eid[bad] == -1 and np.count_nonzero(eid < 0) == 1
    # the same input in the oracle: that particle, and only it, unsolved
    orc = O.OracleRun(p, rc)
    assert orc.initialize() == 1
    st = orc.get_int("eos_status")
    assert st[bad] < 0 and np.count_nonzero(st < 0) == 1


def test_negative_energy_has_no_solution():
    p, rc = ics.gubser_2d(n_side=24)
    p.e[7] = -1.0
    g = api.GpuHydro(rc)
    g.load(p)
    _expect(EOS, g.initialize)
    assert g.get_int("eos_id")[7] == -1
    orc = O.OracleRun(p, rc)
    assert orc.initialize() == 1 and orc.get_int("eos_id")[7] == -1


def test_unsolvable_charge_freezes_the_particle_and_retries_at_zero_charge():
    # conformal-diagonal EoS: a density far above what the energy can carry
    # has no solution; the reference freezes the particle and solves it at
    # zero charge (src/sph_workstation.cpp:1825-1848), and so do both here
    p, rc = ics.hotspots_2d(n_side=24, n_hot=3, seed=2)
    k = 50
    p.rhoB[k] = 1e4 * p.e[k]
    g = api.GpuHydro(rc)
    g.load(p)
    g.initialize()
    orc = O.OracleRun(p, rc)
    assert orc.initialize() == 0
    fz = g.get_int("freeze")
    assert fz[k] == 4
    assert np.array_equal(fz, orc.get_int("freeze"))
    # the state after the initial smoothing agrees with the oracle's
    for f in ("s", "T", "muB", "sigma"):
        a, b = g.get(f), orc.get(f)
        assert np.max(np.abs(a - b) / (np.abs(b) + 1e-6 * np.max(np.abs(b)))) < 1e-10, f


def test_non_finite_position_is_rejected_at_load():
    p, rc = ics.hotspots_2d(n_side=24, n_hot=3, seed=2)
    p.x[3] = np.inf
    g = api.GpuHydro(rc)
    msg = _expect(INVALID, g.load, p)
    assert "particle 3" in msg


def test_batch_inversion_reports_unsolvable_rows():
    rc = ics.RunConfig(eos_kind=1, thermo_mode=1)
    rng = np.random.default_rng(4)
    n = 256
    T = rng.uniform(0.5, 2.0, n)
    x = np.column_stack([T, 0.1 * T, 0.0 * T, 0.04 * T])
    g = api.GpuHydro(rc)
    fw = g.eos_thermo(0, x)
    tgt = np.column_stack([fw[:, 5], fw[:, 2], fw[:, 3], fw[:, 4]])
    tgt[10, 0] = -1.0            # negative energy
    tgt[20, 0] = np.nan          # not a number
    tgt[30, 1] = 1e6             # a charge the energy cannot carry
    seeds = np.tile([580 / 197.3269804, 0, 0, 0], (n, 1))
    xg, _, stg, _ = g.eos_invert(0, tgt, seeds)
    xo, _, sto, _ = O.eos_invert_batch(rc, 0, tgt, seeds=seeds)
    assert set(np.flatnonzero(stg < 0)) == {10, 20, 30}
    assert np.array_equal(stg, sto)
    ok = stg >= 0
    assert np.max(np.abs(xg[ok, 0] / x[ok, 0] - 1.0)) < 1e-10


def test_negative_entropy_is_reported_first():
    # a bulk pressure 1000x the thermal one in an expanding flow drives the
    # entropy of the outer particles below zero in the first substep; the
    # EoS failures that follow at those particles are counted after it
    p, rc = ics.gubser_2d(n_side=40)
    rc = dataclasses.replace(rc, zeta_over_s=0.2, zeta_mode=1)
    trace = 1000.0 * p.e / 3.0
    g = api.GpuHydro(rc)
    g.load(p)
    g.set_initial_viscous(trace=trace)
    g.initialize()
    msg = _expect(NEG_ENTROPY, g.step, 1)
    assert "particles with negative entropy" in msg
    orc = O.OracleRun(p, rc)
    orc.set_initial_viscous(trace=trace)
    assert orc.initialize() == 0
    orc.step(1)
    assert np.count_nonzero(orc.get_int("eos_status") == -2) > 0


def test_server_refuses_an_event_over_its_budget():
    p, rc = ics.hotspots_2d(n_side=100, n_hot=3, seed=2)
    q, qrc = ics.hotspots_2d(n_side=8, n_hot=2, seed=2)
    budget = 2 * api.estimate_device_bytes(qrc, q.n)
    assert api.estimate_device_bytes(rc, p.n) > budget
    srv = api.Server(hbm_budget_bytes=budget)
    try:
        with pytest.raises(api.CcakeError) as ei:
            srv.submit(p, rc, rc.t0 + 0.01)
        assert ei.value.code == CAPACITY
        # a small event still runs on the same server
        t = srv.submit(q, qrc, qrc.t0 + 0.005)
        srv.wait_all()
        assert srv.poll(t)["state"] == "done"
    finally:
        srv.close()


@pytest.mark.parametrize("damage", ["truncated", "garbled", "header", "huge_header", "flat_axis"])
def test_damaged_thermo_dat_is_rejected(tmp_path, damage):
    n, lo, d, f = eos_table.synthetic_table(nT=7, nmu=5)
    path = tmp_path / "thermo.dat"
    eos_table.write_thermo_dat(path, n, lo, d, f, normalize_by_T=True)
    lines = path.read_text().splitlines()
    if damage == "truncated":
        lines = lines[:-3]
    elif damage == "garbled":
        parts = lines[5].split()
        parts[7] = "x1.0"
        lines[5] = " ".join(parts)
    elif damage == "header":
        lines[0] = "7 5 5"
    elif damage == "huge_header":
        lines[0] = "100000 100000 100000 100000"
    else:   # every T the same: no increasing axis
        for i in range(1, len(lines)):
            parts = lines[i].split()
            parts[0] = "100.0"
            lines[i] = " ".join(parts)
    path.write_text("\n".join(lines) + "\n")
    conf5, cdiag5 = eos_table.fallback_scales()
    g = api.GpuHydro(ics.RunConfig(eos_kind=2, thermo_mode=1))
    _expect(INVALID, g.set_eos_table_file, path, True, conf5, cdiag5)
    # the context is still usable: an intact table loads
    eos_table.write_thermo_dat(path, n, lo, d, f, normalize_by_T=True)
    g.set_eos_table_file(path, True, conf5, cdiag5)
