"""CPU restatement of the reference's tabulated-EoS loader (test
infrastructure only): EoS_table::EoS_table (src/eos_table.cpp:14-100) over
InterpolatorND<4>::load_data_from_dat and construct_interpolant
(src/interpolatorND.cpp:125-228).

- line 1: the 4 grid sizes; each further line: 4 grid coordinates, then the
  fields (p s B S Q e cs2 chiBB chiQQ chiSS chiBQ chiBS chiQS chiTB chiTQ
  chiTS chiTT), nodes in file order (row-major, last axis fastest);
- the axes are multiplied by 1/hbarc (MeV -> fm^-1); each axis' grid is
  min + i * (max - min) / (n - 1) of the rescaled column;
- normalize_by_T: p, e x T^4; s, B, S, Q x T^3; the ten chi x T^2, with T the
  row's rescaled temperature; otherwise the fields x (1/hbarc)^k for MeV^k.
"""
import numpy as np

HBARC_MEV = 197.3269804
POWERS = (4, 3, 3, 3, 3, 4, 0, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2)


def read_thermo_dat(path, normalize_by_T=True):
    with open(path) as fh:
        n = np.array([int(v) for v in fh.readline().split()], dtype=np.int32)
        data = np.loadtxt(fh, dtype=np.float64, ndmin=2)
    grid = data[:, :4] * (1.0 / HBARC_MEV)
    fields = data[:, 4:].copy()
    lo = grid.min(axis=0)
    hi = grid.max(axis=0)
    d = np.where(n > 1, (hi - lo) / np.maximum(n - 1.0, 1.0), 0.0)
    pw = np.array(POWERS, dtype=np.float64)
    if normalize_by_T:
        fields *= grid[:, :1] ** pw
    else:
        hc1 = 1.0 / HBARC_MEV
        fields *= np.array([hc1 ** k for k in POWERS])
    return n, lo, d, fields
