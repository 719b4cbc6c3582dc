"""The reference's thermo.dat table format: the writer against the CPU
restatement of the reference's loader (oracle/thermo_dat.py), both unit
conventions, and the library's reader against it on the GPU."""
import ctypes

import numpy as np
import pytest

from ccake_gb300 import eos_table, ics
import oracle_py as O
import thermo_dat


@pytest.mark.parametrize("normalize", [True, False])
def test_write_read_round_trip(tmp_path, normalize):
    n, lo, d, f = eos_table.synthetic_table(nT=9, nmu=5)
    path = tmp_path / "thermo.dat"
    eos_table.write_thermo_dat(path, n, lo, d, f, normalize_by_T=normalize)
    with open(path) as fh:
        assert fh.readline().split() == ["9", "5", "5", "5"]
        assert len(fh.readline().split()) == 21
    n2, lo2, d2, f2 = thermo_dat.read_thermo_dat(path, normalize_by_T=normalize)
    assert np.array_equal(n2, n)
    assert np.allclose(lo2, lo, rtol=1e-14, atol=1e-15)
    assert np.allclose(d2, d, rtol=1e-13)
    assert np.allclose(f2, f, rtol=1e-13, atol=1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("normalize", [True, False])
def test_library_reader_matches_reference_loader(tmp_path, normalize):
    from ccake_gb300 import api
    n, lo, d, f = eos_table.synthetic_table(nT=13, nmu=7)
    eos_table.write_thermo_dat(tmp_path / "thermo.dat", n, lo, d, f, normalize_by_T=normalize)
    conf5, cdiag5 = eos_table.fallback_scales()
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    g = api.GpuHydro(rc)
    g.set_eos_table_file(tmp_path, normalize, conf5, cdiag5)   # a directory holding thermo.dat
    n2, lo2, d2, f2 = thermo_dat.read_thermo_dat(tmp_path / "thermo.dat", normalize_by_T=normalize)
    ot = O.OracleTable(n2, lo2, d2, f2, conf5, cdiag5)
    cfg = O.make_config(rc)
    x = eos_table.sample_states(500, seed=8)
    og = g.eos_thermo(0, x)
    for i in range(x.shape[0]):
        o = np.zeros(17)
        O.lib().orc_eos_full_thermo(ctypes.byref(cfg), ot.h, 0, O._dp(x[i].copy()), O._dp(o))
        assert np.allclose(og[i], o, rtol=1e-12, atol=1e-12 * np.abs(o).max()), i
