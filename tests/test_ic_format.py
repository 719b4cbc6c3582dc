"""The "ccake" initial-condition reader of the library (ccake_ic_read_ccake)
against the oracle's restatement of src/BSQHydro.cpp:206-425, on files
written here: bit-exact columns, the header grid, skipped lines, the energy
cutoff, entropy input, disabled charges, initial diffusion and the error
cases. Host code only (no GPU)."""
import math

import numpy as np
import pytest

from ccake_gb300 import api
import ic_format as R


def gubser_lines(n_side=24, seed=1, ncol=17):
    """A Gubser-flow profile (the ideal solution's energy density and
    velocity at tau0 = 1 fm/c, q = 1 fm^-1) with random charges and shear,
    in the file format's columns."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-3.0, 3.0, n_side)
    out = []
    for x in xs:
        for y in xs:
            r = math.hypot(x, y)
            e = 80.0 * 2.0 ** (8.0 / 3.0) / (1.0 + 2.0 * (1.0 + r * r) + (1.0 - r * r) ** 2) ** (4.0 / 3.0) * 0.1973269804
            k = math.atanh(2.0 * r / (2.0 + r * r))
            ux, uy = (math.sinh(k) * x / r, math.sinh(k) * y / r) if r > 0 else (0.0, 0.0)
            row = [x, y, 0.0, e, *rng.normal(size=3) * 0.1, ux, uy, 0.0, *rng.normal(size=7) * 1e-3]
            row += list(rng.normal(size=ncol - 17) * 1e-2)
            out.append(" ".join(f"{v:.17g}" for v in row))
    return out


def write(path, lines, header="#0 0.25 0.25 0.1 0 -3.0 -3.0 -0.1"):
    with open(path, "w") as fh:
        fh.write(header + "\n")
        for k, l in enumerate(lines):
            fh.write(l + "\n")
            if k % 97 == 5:
                fh.write("\n   \n# a comment line\n")
    return str(path)


def compare(path, **kw):
    p, cols, grid = api.read_ccake_ic(path, **kw)
    ref, rgrid = R.read_ccake(path, **kw)
    assert grid == rgrid
    for c in R.COLUMNS:
        assert np.array_equal(cols[c], np.array(ref[c], dtype=np.float64)), c
    assert p.n == len(ref["x"])
    return p, cols


def test_reader_matches_oracle(tmp_path):
    path = write(tmp_path / "ic.dat", gubser_lines())
    p, cols = compare(path)
    assert p.n == 24 * 24
    assert np.array_equal(p.e, cols["e"]) and np.array_equal(p.ux, cols["ux"])
    # GeV/fm^3 -> fm^-4
    assert abs(cols["e"].max() * 0.1973269804 - 80.0 * 2.0 ** (8.0 / 3.0) / 4.0 ** (4.0 / 3.0) * 0.1973269804) < 1.0


def test_energy_cutoff_and_charges(tmp_path):
    path = write(tmp_path / "ic.dat", gubser_lines(seed=2))
    p, cols = compare(path, e_cutoff=0.5, charges=(1, 0, 1))
    assert 0 < p.n < 24 * 24
    assert np.all(cols["e"] * 0.1973269804 > 0.5)
    assert not np.any(cols["rhoS"])


def test_entropy_input(tmp_path):
    path = write(tmp_path / "ic.dat", gubser_lines(seed=3))
    p, cols = compare(path, input_as_entropy=1, e_cutoff=0.2)
    assert p.n > 0


def test_initial_diffusion_columns(tmp_path):
    path = write(tmp_path / "ic.dat", gubser_lines(seed=4, ncol=29))
    p, cols = compare(path, input_initial_diffusion=1, charges=(1, 1, 0))
    assert np.any(cols["qB1"]) and not np.any(cols["qQ2"])


def test_errors(tmp_path):
    with pytest.raises(api.CcakeError):
        api.read_ccake_ic(tmp_path / "missing.dat")
    bad = write(tmp_path / "nohash.dat", gubser_lines(n_side=4), header="0 0.25 0.25 0.1 0 -3 -3 -0.1")
    with pytest.raises(api.CcakeError):
        api.read_ccake_ic(bad)
    short = write(tmp_path / "short.dat", gubser_lines(n_side=4) + ["1 2 3"])
    with pytest.raises(api.CcakeError):
        api.read_ccake_ic(short)
    with pytest.raises(ValueError):
        R.read_ccake(short)
