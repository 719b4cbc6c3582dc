"""Synthetic tabulated 4-D equation of state (fm units), the EoS-inversion
stress-test table.

Pressure, natural units (T and mu in fm^-1, p in fm^-4; the GeV constants
below are divided by hbar c):

    p(T, muB, muS, muQ) = [a T^4 + b T^2 (muB^2 + muS^2 + muQ^2) + c muB^4] S(T)
                          + h exp(-m/T) [T^4 + k T^2 (muB^2 + muS^2 + muQ^2)]
    S(T) = (1 + tanh((T - Tc)/delta)) / 2

a = 5.3, b = 0.5, c = 0.05, Tc = 0.155 GeV, delta = 0.02 GeV (the QGP part
as specified for this table); the second term is a Boltzmann-suppressed
hadron-gas pressure with h = 2, m = 0.4 GeV, k = 1. Every field of a node is
exact: s = dp/dT, rho_i = dp/dmu_i, e = T s + sum mu_i rho_i - p, the ten
second derivatives (susceptibilities), and the adiabatic sound speed
cs^2 = s^2 v^T H^-1 v / w with v = (1, rho_B/s, rho_S/s, rho_Q/s) and H the
Hessian of p in (T, muB, muS, muQ) (d e = (w/s) d s and d p = s v^T d(T, mu)
along d(rho_i/s) = 0).

Grid: T in [0.05, 0.8] GeV (151 points), each mu in [-0.45, 0.45] GeV (41
points), stored in fm^-1. Node layout (reference src/eos_table.cpp:31-35,
include/interpolatorND.h:132-138): (T, muB, muQ, muS) row-major, muS
fastest, 17 fields per node

    p s rhoB rhoS rhoQ e cs2 chiBB chiQQ chiSS chiBQ chiBS chiQS chiTB chiTQ chiTS chiTT
"""
from __future__ import annotations

import numpy as np

HBARC = 0.1973269804    # GeV fm

A_QGP, B_QGP, C_QGP = 5.3, 0.5, 0.05
TC_GEV, DELTA_GEV = 0.155, 0.02
H_HG, M_HG_GEV, K_HG = 2.0, 0.4, 1.0


def thermo(T, mB, mS, mQ):
    """All 17 fields at (T, muB, muS, muQ) in fm^-1 (arrays broadcast);
    returns an array of shape (..., 17) in the node field order."""
    T = np.asarray(T, dtype=np.float64)
    mB, mS, mQ = (np.asarray(v, dtype=np.float64) for v in (mB, mS, mQ))
    Tc, dl = TC_GEV / HBARC, DELTA_GEV / HBARC
    m = M_HG_GEV / HBARC
    M2 = mB * mB + mS * mS + mQ * mQ
    th = np.tanh((T - Tc) / dl)
    S = 0.5 * (1.0 + th)
    S1 = 0.5 * (1.0 - th * th) / dl
    S2 = -(th * (1.0 - th * th)) / (dl * dl)
    a, b, c = A_QGP, B_QGP, C_QGP
    P0 = a * T ** 4 + b * T * T * M2 + c * mB ** 4
    P0T = 4 * a * T ** 3 + 2 * b * T * M2
    P0TT = 12 * a * T * T + 2 * b * M2
    E = H_HG * np.exp(-m / T)
    E1 = E * m / (T * T)
    E2 = E * (m * m / T ** 4 - 2 * m / T ** 3)
    k = K_HG
    Q = T ** 4 + k * T * T * M2
    QT = 4 * T ** 3 + 2 * k * T * M2
    QTT = 12 * T * T + 2 * k * M2
    mu = (mB, mS, mQ)
    p = P0 * S + E * Q
    s = P0T * S + P0 * S1 + E1 * Q + E * QT
    rho = [(2 * b * T * T * mu_i + (4 * c * mB ** 3 if i == 0 else 0.0)) * S + E * 2 * k * T * T * mu_i
           for i, mu_i in enumerate(mu)]
    chi_TT = P0TT * S + 2 * P0T * S1 + P0 * S2 + E2 * Q + 2 * E1 * QT + E * QTT
    # d2p/dT dmu_i
    chi_T = [(4 * b * T * mu_i) * S + (2 * b * T * T * mu_i + (4 * c * mB ** 3 if i == 0 else 0.0)) * S1
             + E1 * 2 * k * T * T * mu_i + E * 4 * k * T * mu_i for i, mu_i in enumerate(mu)]
    diag = 2 * b * T * T * S + E * 2 * k * T * T
    chi_BB = diag + 12 * c * mB * mB * S
    chi_SS = diag
    chi_QQ = diag
    zero = np.zeros_like(p)
    e = T * s + mB * rho[0] + mS * rho[1] + mQ * rho[2] - p
    w = e + p
    # adiabatic sound speed from the Hessian in (T, muB, muS, muQ)
    H = np.empty(p.shape + (4, 4))
    H[..., 0, 0] = chi_TT
    H[..., 0, 1] = H[..., 1, 0] = chi_T[0]
    H[..., 0, 2] = H[..., 2, 0] = chi_T[1]
    H[..., 0, 3] = H[..., 3, 0] = chi_T[2]
    H[..., 1, 1] = chi_BB
    H[..., 2, 2] = chi_SS
    H[..., 3, 3] = chi_QQ
    H[..., 1, 2] = H[..., 2, 1] = zero
    H[..., 1, 3] = H[..., 3, 1] = zero
    H[..., 2, 3] = H[..., 3, 2] = zero
    v = np.stack([np.ones_like(s), rho[0] / s, rho[1] / s, rho[2] / s], axis=-1)
    Hv = np.linalg.solve(H, v[..., None])[..., 0]
    cs2 = s * s * np.sum(v * Hv, axis=-1) / w
    # node order: p s B S Q e cs2 chiBB chiQQ chiSS chiBQ chiBS chiQS chiTB chiTQ chiTS chiTT
    return np.stack([p, s, rho[0], rho[1], rho[2], e, cs2, chi_BB, chi_QQ, chi_SS, zero, zero, zero,
                     chi_T[0], chi_T[2], chi_T[1], chi_TT], axis=-1)


def grid(nT=151, nmu=41, T_range=(0.05, 0.8), mu_max=0.45):
    """Axes (fm^-1) of the table: n, lo, d for (T, muB, muQ, muS)."""
    n = np.array([nT, nmu, nmu, nmu], dtype=np.int32)
    lo = np.array([T_range[0], -mu_max, -mu_max, -mu_max]) / HBARC
    hi = np.array([T_range[1], mu_max, mu_max, mu_max]) / HBARC
    d = (hi - lo) / (n - 1)
    return n, lo, d


def synthetic_table(nT=151, nmu=41, T_range=(0.05, 0.8), mu_max=0.45):
    """(n[4], lo[4], d[4], fields[N, 17]) with N = nT nmu^3, nodes in
    (T, muB, muQ, muS) row-major order, muS fastest. Generated one T plane at
    a time (the full table is 1.4 GB at 151 x 41^3)."""
    n, lo, d = grid(nT, nmu, T_range, mu_max)
    axes = [lo[k] + d[k] * np.arange(n[k]) for k in range(4)]
    plane = nmu ** 3
    fields = np.empty((int(nT) * plane, 17))
    B, Q, S = np.meshgrid(axes[1], axes[2], axes[3], indexing="ij")
    for it, T in enumerate(axes[0]):
        fields[it * plane:(it + 1) * plane] = thermo(np.full(B.shape, T), B, S, Q).reshape(plane, 17)
    return n, lo, d, fields


def fallback_scales():
    """Simple (c, T0, muB0, muQ0, muS0) of the analytic fallbacks behind the
    table: the table's high-T limit p -> a T^4 with unit scales (a fixed
    choice for tests that need one). The reference matches them to the table
    at 1.1 T_FO instead: api.table_fallback_scales, or ``None`` scales in
    GpuHydro.set_eos_table."""
    conf = np.array([A_QGP, 1.0, 1.0, 1.0, 1.0])
    return conf, conf.copy()


def sample_states(n, seed=20251205, T_range=(0.05, 0.8), mu_max=0.45, margin=1e-3):
    """n states drawn uniformly in the table's (T, mu) box (fm^-1), a
    relative margin inside its edges; columns (T, muB, muQ, muS)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo = np.array([T_range[0], -mu_max, -mu_max, -mu_max]) / HBARC
    hi = np.array([T_range[1], mu_max, mu_max, mu_max]) / HBARC
    span = hi - lo
    return lo + span * (margin + (1 - 2 * margin) * rng.uniform(size=(n, 4)))


HBARC_MEV = 197.3269804   # MeV fm (the reference's hbarc_MeVfm)
# powers of T (normalize_by_T) or of MeV (absolute units) per field, file order
FIELD_POWERS = (4, 3, 3, 3, 3, 4, 0, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2)
FIELD_NAMES = ("p", "s", "B", "S", "Q", "e", "cs2", "chiBB", "chiQQ", "chiSS", "chiBQ", "chiBS", "chiQS",
               "chiTB", "chiTQ", "chiTS", "chiTT")


def write_thermo_dat(path, n, lo, d, fields, normalize_by_T=True):
    """Writes a table (fm units, nodes row-major with muS fastest) as the
    reference's thermo.dat: a header line with the 4 grid sizes, then one row
    per node `T muB muQ muS p s B S Q e cs2 chiBB chiQQ chiSS chiBQ chiBS chiQS
    chiTB chiTQ chiTS chiTT` with the axes in MeV and the fields divided by
    T^k (normalize_by_T, T in fm^-1) or in MeV^k (src/eos_table.cpp:14-100,
    src/interpolatorND.cpp:125-168). Values are printed with 17 significant
    digits."""
    n = np.asarray(n, dtype=np.int64)
    lo = np.asarray(lo, dtype=np.float64)
    d = np.asarray(d, dtype=np.float64)
    fields = np.asarray(fields, dtype=np.float64)
    axes = [lo[k] + d[k] * np.arange(n[k]) for k in range(4)]
    grid = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 4)
    pw = np.array(FIELD_POWERS, dtype=np.float64)
    if normalize_by_T:
        f = fields / grid[:, :1] ** pw
    else:
        f = fields * HBARC_MEV ** pw
    with open(path, "w") as fh:
        fh.write(" ".join(str(int(v)) for v in n) + "\n")
        np.savetxt(fh, np.hstack([grid * HBARC_MEV, f]), fmt="%.17g")
