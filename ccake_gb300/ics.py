"""Synthetic initial conditions and run configurations for the SPH hot path.

Every workload here is generated in memory with a seeded generator; no dataset
is read. Units are the reference's internal ones: positions in fm (eta is
dimensionless), energy density in fm^-4 (GeV/fm^3 divided by hbar*c),
charge densities in fm^-3, temperatures in fm^-1.

Workloads
---------
gubser_2d       ideal 2+1-D Gubser flow, conformal EoS (the analytic-oracle case)
hotspots_2d     viscous 2+1-D BSQ run, 30 Gaussian hot spots, conformal-diagonal EoS
hotspots_3d     viscous 3+1-D Milne run, tabulated EoS (see ``eos_table``)
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

HBARC_GEVFM = 0.1973269804   # include/constants.h:16 of the reference
HBARC_MEVFM = 197.3269804

# Reference conformal constant: c = pi^2 (2 (Nc^2 - 1) + 3.5 Nc Nf) / 90 with
# Nc = 3, Nf = 2.5 (src/eos_initialization.cpp:226-229); p = c T^4.
C_REFERENCE = math.pi ** 2 * (2.0 * (3.0 * 3.0 - 1.0) + 3.5 * 3.0 * 2.5) / 90.0


@dataclasses.dataclass
class RunConfig:
    """Mirror of the C ``ccake_config`` (and of the oracle's ``Config``)."""
    dim: int = 2
    coord: int = 0                 # 0 Milne ("hyperbolic"), 1 Cartesian
    eos_kind: int = 0              # 0 conformal, 1 conformal_diagonal, 2 table
    using_shear: int = 0
    using_vorticity: int = 0
    shear_relax_mode: int = 0      # 0 default max(5 eta/w, 0.005), 1 "Gubser" 5 eta/w
    zeta_mode: int = 1             # 0 default, 1 constant, 2 cs2-dependent, 3 peaked
    factorized_kernel: int = 0
    input_as_entropy: int = 0
    modulate_zeta_with_tanh: int = 0
    thermo_mode: int = 0           # 0 reference derivative chain, 1 exact Hessian inverse
    precision: int = 0             # 0 FP64 throughout, 1 FP32 compensated pair loops (GPU only)
    hT: float = 0.1
    hEta: float = 0.1
    t0: float = 1.0
    dt: float = 0.001
    eos_c: float = C_REFERENCE
    eos_T0: float = 1.0
    eos_muB0: float = 1.0
    eos_muQ0: float = 1.0
    eos_muS0: float = 1.0
    eta_over_s: float = 0.0
    zeta_over_s: float = 0.0
    zeta_cs2_A: float = 1.67552
    zeta_cs2_p: float = 2.0
    zeta_peak_T: float = 0.16 / HBARC_GEVFM
    zeta_peak_width: float = 0.02 / HBARC_GEVFM
    xmin: float = -5.0
    ymin: float = -5.0
    etamin: float = -0.1
    freeze_out_T: float = 150.0 / HBARC_MEVFM
    skin_frac: float = 0.0         # candidate-list skin / 2h (0: 0.1), GPU only
    particlization: int = 0        # freeze-out status machine after every step
    surface: int = 0               # with particlization: the freeze-out hypersurface rows
    # diffusion sector (FP64 form, Milne coordinates)
    using_diffusion: int = 0
    diffusion_mode: int = 0        # 0 constant_over_T2, 2 kappaB_coth
    diffusion_relax_mode: int = 0  # 0 tau_q = 0.2/T, 1 tau_q = C_B/T (kappaB_coth)
    diffusion_regulator: int = 0   # regulate_diffusion (PhysRevC.98.034916 Eqs. C6-C8)
    critical_scaling_diffusion: int = 0
    kappa_over_T2: tuple = (0.0,) * 9   # row-major 3x3 over (B, S, Q)
    C_B: float = 0.0
    reg_chi0: float = 10.0
    reg_e0: float = 0.1            # GeV/fm^3
    reg_xi0: float = 0.01          # GeV/fm^3
    reg_rq_max: float = 1.0
    crit_T: float = 150.0          # MeV
    crit_muB: float = 350.0        # MeV
    crit_wT: float = 30.0          # MeV
    crit_wmuB: float = 50.0        # MeV
    # second-order transport coefficients: 0 the reference's *_DEFAULT
    # function, 1 "israel-stewart" (delta_pipi, delta_PiPi only), 2 disabled
    delta_pipi_mode: int = 0
    tau_pipi_mode: int = 0
    lambda_piPi_mode: int = 0
    phi6_mode: int = 0
    phi7_mode: int = 0
    delta_PiPi_mode: int = 0
    lambda_Pipi_mode: int = 0
    phi1_mode: int = 0
    phi3_mode: int = 0
    # initial e -> (T, mu) inversion: 0 the reference's seeds, 2 the learned
    # seed (trained network, table EoS) first
    seed_mode: int = 0
    # refuse table solutions with a chemical potential above 3.5 T
    restrict_mu_T_ratios: int = 0


@dataclasses.dataclass
class Particles:
    """Host struct-of-arrays input (the reference's ccake IC columns)."""
    x: np.ndarray
    y: np.ndarray
    eta: np.ndarray
    e: np.ndarray          # energy density, fm^-4 (or entropy density when input_as_entropy)
    rhoB: np.ndarray
    rhoS: np.ndarray
    rhoQ: np.ndarray
    ux: np.ndarray
    uy: np.ndarray
    ueta: np.ndarray

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def take(self, idx) -> "Particles":
        return Particles(*(getattr(self, f.name)[idx] for f in dataclasses.fields(self)))


def lattice_2d(nx: int, ny: int, dx: float, xmin: float, ymin: float):
    """Lattice points x_i = xmin + i*dx in FP64 (row-major, x fastest)."""
    i = np.arange(nx, dtype=np.float64)
    j = np.arange(ny, dtype=np.float64)
    xs = xmin + i * dx
    ys = ymin + j * dx
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    return X.ravel().copy(), Y.ravel().copy()


def gubser_temperature(tau, r, q=1.0, That0=1.2):
    """Ideal Gubser temperature (fm^-1), BASELINE config 1 formula."""
    num = (That0 / tau ** (1.0 / 3.0)) * (2.0 * q) ** (2.0 / 3.0)
    den = (1.0 + 2.0 * q * q * (tau * tau + r * r) + q ** 4 * (tau * tau - r * r) ** 2) ** (1.0 / 3.0)
    return num / den


def gubser_ur(tau, r, q=1.0):
    """Radial spatial four-velocity u^r = sinh(kappa), tanh(kappa) = v^r
    (utilities/ideal_gubser_ic_generator.py:31-36 of the reference)."""
    kap = np.arctanh(2.0 * q * q * tau * r / (1.0 + q * q * tau * tau + q * q * r * r))
    return np.sinh(kap)


def gubser_2d(n_side=200, dx=0.05, h=0.1, tau0=1.0, dt=0.001, c_e=15.6269, q=1.0, That0=1.2):
    """Config 1: ideal Gubser flow on an n_side^2 lattice over [-5, 5)^2.

    ``c_e`` is the coefficient of e = c_e T^4; the conformal EoS is set to
    p = (c_e/3) T^4 so the analytic solution applies. Pass ``c_e = 3*C_REFERENCE``
    for the reference's own constant.
    """
    xmin = -0.5 * n_side * dx
    x, y = lattice_2d(n_side, n_side, dx, xmin, xmin)
    r = np.sqrt(x * x + y * y)
    T = gubser_temperature(tau0, r, q, That0)
    e = c_e * T ** 4
    ur = gubser_ur(tau0, r, q)
    with np.errstate(invalid="ignore", divide="ignore"):
        ux = np.where(r > 0, ur * x / np.where(r > 0, r, 1.0), 0.0)
        uy = np.where(r > 0, ur * y / np.where(r > 0, r, 1.0), 0.0)
    z = np.zeros_like(x)
    p = Particles(x, y, z.copy(), e, z.copy(), z.copy(), z.copy(), ux, uy, z.copy())
    cfg = RunConfig(dim=2, eos_kind=0, using_shear=0, hT=h, t0=tau0, dt=dt,
                    eos_c=c_e / 3.0, xmin=xmin, ymin=xmin, etamin=-0.1, zeta_mode=1,
                    zeta_over_s=0.0, eta_over_s=0.0)
    return p, cfg


class GubserIS:
    """Semi-analytic Gubser flow of Israel-Stewart theory with constant
    eta/s (Marrochio, Noronha, Denicol, Luzum, Jeon, Gale,
    PhysRevC.91.014903; the reference tabulates it with
    misc/Gubser_checks/ac/Gubser_semi-analytical_tabulator.wls).

    In de Sitter time rho = -asinh((1 - tau^2 + r^2) / (2 tau)) the flow
    reduces to two ODEs for That(rho) and the normalised shear pibar(rho):
        That'/That + (2/3) tanh rho = (1/3) pibar tanh rho
        c (eta/s)/That (pibar' + (4/3) pibar^2 tanh rho) + pibar
            = (4/3) (eta/s)/That tanh rho
    with That(0) = 1.2, pibar(0) = 0 and tau_pi = c eta/(e + p), c = 5. They
    are integrated here in both directions from rho = 0 (scipy DOP853, rtol
    1e-12) and mapped back:
        T = That(rho)/tau,  u^r = sinh(atanh(2 tau r / (1 + tau^2 + r^2))),
        pihat = (4/3) alpha That^4 pibar,  alpha = 3 c_ref (e = alpha T^4),
        pi^{ij} = -(1/2) tau^-4 (delta^{ij} + x^i x^j / r^2 (u^r)^2) pihat,
        tau^2 pi^{eta eta} = pihat / tau^4.
    Units are the library's: fm^-1 for T, fm^-4 for pi.
    """

    def __init__(self, eta_over_s=0.2, c_tau=5.0, That0=1.2, rho_range=(-8.0, 4.0)):
        from scipy.integrate import solve_ivp
        self.eta_over_s, self.c_tau = eta_over_s, c_tau
        self.alpha = 3.0 * C_REFERENCE

        def rhs(r, y):
            T, pb = y
            th = math.tanh(r)
            return [T * (pb * th / 3.0 - 2.0 * th / 3.0),
                    (4.0 / 3.0 * eta_over_s / T * th - pb) * T / (c_tau * eta_over_s) - 4.0 / 3.0 * pb * pb * th]

        kw = dict(method="DOP853", rtol=1e-12, atol=1e-14, dense_output=True)
        self._neg = solve_ivp(rhs, (0.0, rho_range[0]), [That0, 0.0], **kw).sol
        self._pos = solve_ivp(rhs, (0.0, rho_range[1]), [That0, 0.0], **kw).sol

    def hat(self, rho):
        rho = np.asarray(rho, dtype=np.float64)
        out = np.empty((2,) + rho.shape)
        m = rho < 0
        out[:, m] = self._neg(rho[m])
        out[:, ~m] = self._pos(rho[~m])
        return out

    def fields(self, tau, x, y):
        """T, u^x, u^y, pi^xx, pi^yy, pi^xy, tau^2 pi^{eta eta} at (tau, x, y)."""
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        r = np.sqrt(x * x + y * y)
        rho = -np.arcsinh((1.0 - tau * tau + r * r) / (2.0 * tau))
        Th, pb = self.hat(rho)
        ur = np.sinh(np.arctanh(2.0 * tau * r / (1.0 + tau * tau + r * r)))
        rs = np.where(r > 0, r, 1.0)
        cx, cy = np.where(r > 0, x / rs, 0.0), np.where(r > 0, y / rs, 0.0)
        pih = 4.0 / 3.0 * self.alpha * Th ** 4 * pb
        f = -0.5 / tau ** 4 * pih
        return dict(T=Th / tau, ux=cx * ur, uy=cy * ur, pixx=f * (1.0 + cx * cx * ur * ur),
                    piyy=f * (1.0 + cy * cy * ur * ur), pixy=f * cx * cy * ur * ur, t2pietaeta=pih / tau ** 4)


def gubser_viscous_2d(n_side=281, dx=0.05, h=0.1, tau0=1.0, dt=0.001, eta_over_s=0.2, solution=None):
    """Viscous Gubser flow (Israel-Stewart, eta/s = 0.2, tau_pi = 5 eta/w) on
    an n_side^2 lattice centred on the origin, at tau0 = 1 fm/c: T, u^i and
    pi^{ij} of the semi-analytic solution (``GubserIS``), conformal EoS
    e = 3p = 3 c_ref T^4 (the reference's constant). Returns (particles,
    config, pi[6, n] in the order xx xy xeta yy yeta etaeta for
    ``set_initial_viscous``)."""
    sol = solution or GubserIS(eta_over_s=eta_over_s)
    xmin = -0.5 * (n_side - 1) * dx
    x, y = lattice_2d(n_side, n_side, dx, xmin, xmin)
    f = sol.fields(tau0, x, y)
    e = 3.0 * C_REFERENCE * f["T"] ** 4
    z = np.zeros_like(x)
    p = Particles(x, y, z.copy(), e, z.copy(), z.copy(), z.copy(), f["ux"], f["uy"], z.copy())
    pi = np.zeros((6, x.shape[0]))
    pi[0], pi[1], pi[3] = f["pixx"], f["pixy"], f["piyy"]
    pi[5] = f["t2pietaeta"] / tau0 ** 2
    # the reference's viscous Gubser settings (input/config_visc_gubser.yaml):
    # delta_pipi "default" (4/3 tau_pi), tau_pipi, lambda_piPi, phi6 and phi7
    # "disabled" -- the Israel-Stewart equations the solution solves
    cfg = RunConfig(dim=2, eos_kind=0, using_shear=1, shear_relax_mode=1, eta_over_s=eta_over_s,
                    zeta_mode=1, zeta_over_s=0.0, hT=h, t0=tau0, dt=dt, eos_c=C_REFERENCE,
                    xmin=xmin, ymin=xmin, etamin=-0.1, delta_pipi_mode=0, tau_pipi_mode=2,
                    lambda_piPi_mode=2, phi6_mode=2, phi7_mode=2)
    return p, cfg, pi


def hotspots_2d(n_side=400, dx=0.05, h=0.1, n_hot=30, sigma=0.4, seed=20251203, tau0=1.0,
                dt=0.001, eta_over_s=0.08, floor_GeV=0.01, peak_range=(5.0, 50.0), rhoS_frac=0.0):
    """Config 2: 30 Gaussian hot spots (sigma 0.4 fm), centres ~ N(0, 3 fm),
    peaks ~ U[5, 50] GeV/fm^3, plus a uniform floor of ``floor_GeV`` GeV/fm^3
    so that every lattice particle carries matter. rhoB = e[GeV/fm^3]/20 fm^-3,
    rhoS = 0, rhoQ = 0.4 rhoB. Conformal-diagonal EoS with the reference
    constants, eta/s = 0.08 with tau_pi = 5 eta/w ("Gubser"), zeta = 0, u = 0.
    Generator: numpy PCG64 with the given seed.

    ``rhoS_frac`` != 0 gives the event strangeness, rhoS = rhoS_frac * rhoB
    * cos(x / 1 fm): a density that changes sign across the event, so that
    all four densities (and a strangeness chemical potential of either sign)
    are exercised.

    The enthalpy derivatives use the exact inverse of the susceptibility
    matrix (``thermo_mode=1``): with two non-zero charges the reference's
    Schur-complement chain divides by its 1e-25 cross-susceptibility
    placeholders for this EoS and returns dw/drho_B ~ -1e20, after which the
    evolution is not finite.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    cx = rng.normal(0.0, 3.0, n_hot)
    cy = rng.normal(0.0, 3.0, n_hot)
    amp = rng.uniform(peak_range[0], peak_range[1], n_hot)
    xmin = -0.5 * n_side * dx
    x, y = lattice_2d(n_side, n_side, dx, xmin, xmin)
    eG = np.full_like(x, floor_GeV)
    for k in range(n_hot):
        eG += amp[k] * np.exp(-((x - cx[k]) ** 2 + (y - cy[k]) ** 2) / (2.0 * sigma * sigma))
    rhoB = eG / 20.0
    rhoQ = 0.4 * rhoB
    rhoS = rhoS_frac * rhoB * np.cos(x)
    z = np.zeros_like(x)
    p = Particles(x, y, z.copy(), eG / HBARC_GEVFM, rhoB, rhoS, rhoQ, z.copy(), z.copy(), z.copy())
    cfg = RunConfig(dim=2, eos_kind=1, using_shear=1 if eta_over_s > 1e-10 else 0,
                    shear_relax_mode=1, thermo_mode=1, zeta_mode=1, zeta_over_s=0.0, eta_over_s=eta_over_s,
                    hT=h, t0=tau0, dt=dt, xmin=xmin, ymin=xmin, etamin=-0.1)
    return p, cfg


def hotspots_3d(n_xy=120, n_eta=100, dx=0.1, deta=0.06, h=0.2, n_hot=30, sigma_perp=0.4, sigma_eta=0.5,
                plateau=1.5, tail=1.0, seed=20251204, tau0=1.0, dt=0.001, eta_over_s=0.08, floor_GeV=0.01,
                peak_range=(5.0, 50.0), eos_kind=1, zeta_over_s=0.0):
    """Config 4 lattice: (x, y, eta_s) grid, 30 hot spots with sigma_perp = 0.4 fm
    and sigma_eta = 0.5 (centres ~ N(0, 3 fm) in x, y and ~ U[-plateau, plateau]
    in eta), multiplied by a longitudinal plateau of half-width 1.5 with
    Gaussian tails of width 1, plus the floor; charges as in hotspots_2d.
    Milne coordinates, non-factorised 3-D kernel on (x, y, eta) as in the
    reference's default (src/kernel.cpp:34-84). ``eos_kind`` 1 is the
    conformal-diagonal EoS; the tabulated EoS of the 3+1-D benchmark is 2.
    ``zeta_over_s`` > 0 adds bulk viscosity zeta/s peaked at T = 0.16 GeV
    (Gaussian of width 0.02 GeV, zeta_mode 3) with that peak value.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    cx = rng.normal(0.0, 3.0, n_hot)
    cy = rng.normal(0.0, 3.0, n_hot)
    ce = rng.uniform(-plateau, plateau, n_hot)
    amp = rng.uniform(peak_range[0], peak_range[1], n_hot)
    xmin = -0.5 * n_xy * dx
    emin = -0.5 * n_eta * deta
    xs = xmin + dx * np.arange(n_xy, dtype=np.float64)
    es = emin + deta * np.arange(n_eta, dtype=np.float64)
    E, Y, X = np.meshgrid(es, xs, xs, indexing="ij")
    x, y, eta = X.ravel().copy(), Y.ravel().copy(), E.ravel().copy()
    prof = np.where(np.abs(eta) <= plateau, 1.0, np.exp(-((np.abs(eta) - plateau) ** 2) / (2.0 * tail * tail)))
    eG = np.zeros_like(x)
    for k in range(n_hot):
        eG += amp[k] * np.exp(-((x - cx[k]) ** 2 + (y - cy[k]) ** 2) / (2.0 * sigma_perp ** 2)
                              - (eta - ce[k]) ** 2 / (2.0 * sigma_eta ** 2))
    eG = eG * prof + floor_GeV
    rhoB = eG / 20.0
    rhoQ = 0.4 * rhoB
    z = np.zeros_like(x)
    p = Particles(x, y, eta, eG / HBARC_GEVFM, rhoB, z.copy(), rhoQ, z.copy(), z.copy(), z.copy())
    cfg = RunConfig(dim=3, eos_kind=eos_kind, using_shear=1 if eta_over_s > 1e-10 else 0,
                    shear_relax_mode=1, thermo_mode=1, zeta_mode=3 if zeta_over_s > 0 else 1,
                    zeta_over_s=zeta_over_s, eta_over_s=eta_over_s,
                    hT=h, hEta=h, t0=tau0, dt=dt, xmin=xmin, ymin=xmin, etamin=emin)
    return p, cfg
