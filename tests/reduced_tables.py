"""Tables with frozen chemical-potential axes for the reduced modes of the
reference's root finder and derivatives (src/rootfinder.cpp:447-491,
src/eos.cpp:129-141, src/eos_derivatives.cpp:33-260): the synthetic
stress-test EoS of ccake_gb300.eos_table on a T-only grid (one node at
muB = muQ = muS = 0) and a baryon-only grid (one node at muQ = muS = 0)."""
import numpy as np

import fallback_scales as FS
from ccake_gb300 import eos_table, ics

NT, NMU = 76, 21


def reduced_table(kind):
    """(n, lo, d, fields, conf5, cdiag5) of the T-only ("T") or the
    baryon-only ("B") table, fallback scales matched as the reference does."""
    n, lo, d = eos_table.grid(NT, NMU)
    axT = lo[0] + d[0] * np.arange(NT)
    if kind == "T":
        nn = np.array([NT, 1, 1, 1], dtype=np.int32)
        llo = np.array([lo[0], 0.0, 0.0, 0.0])
        dd = np.array([d[0], 1.0, 1.0, 1.0])
        z = np.zeros_like(axT)
        f = eos_table.thermo(axT, z, z, z).reshape(NT, 17)
    else:
        axB = lo[1] + d[1] * np.arange(NMU)
        TT, BB = np.meshgrid(axT, axB, indexing="ij")
        nn = np.array([NT, NMU, 1, 1], dtype=np.int32)
        llo = np.array([lo[0], lo[1], 0.0, 0.0])
        dd = np.array([d[0], d[1], 1.0, 1.0])
        z = np.zeros_like(TT)
        f = eos_table.thermo(TT, BB, z, z).reshape(NT * NMU, 17)
    conf5, cdiag5 = FS.reference_fallback_scales(nn, llo, dd, f, ics.RunConfig().freeze_out_T)
    return nn, llo, dd, np.ascontiguousarray(f), conf5, cdiag5


def reduced_states(kind, n, seed):
    """n states on the table's grid lines at T in [0.2, 0.79] GeV (where this
    EoS is stable); baryon-only states with muB in [-0.4, 0.4] GeV. Columns
    (T, muB, muQ, muS), fm^-1."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = np.zeros((n, 4))
    x[:, 0] = rng.uniform(0.2, 0.79, n) / eos_table.HBARC
    if kind == "B":
        x[:, 1] = rng.uniform(-0.4, 0.4, n) / eos_table.HBARC
    return x
