"""ctypes wrapper of the CPU oracle library (oracle/_build/libccake_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libccake_oracle.so")


class Config(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "dim", "coord", "eos_kind", "using_shear", "using_vorticity", "shear_relax_mode",
        "zeta_mode", "factorized_kernel", "input_as_entropy", "modulate_zeta_with_tanh",
        "thermo_mode", "pad1")] + [(n, ctypes.c_double) for n in (
        "hT", "hEta", "t0", "dt", "eos_c", "eos_T0", "eos_muB0", "eos_muQ0", "eos_muS0",
        "eta_over_s", "zeta_over_s", "zeta_cs2_A", "zeta_cs2_p", "zeta_peak_T",
        "zeta_peak_width", "xmin", "ymin", "etamin", "freeze_out_T")] + [
        ("particlization", ctypes.c_int32), ("surface", ctypes.c_int32)] + [
        (n, ctypes.c_int32) for n in ("using_diffusion", "diffusion_mode", "diffusion_relax_mode",
                                      "diffusion_regulator", "critical_scaling_diffusion", "pad2")] + [
        ("kappa_over_T2", ctypes.c_double * 9)] + [(n, ctypes.c_double) for n in (
        "C_B", "reg_chi0", "reg_e0", "reg_xi0", "reg_rq_max", "crit_T", "crit_muB", "crit_wT", "crit_wmuB")] + [
        (n, ctypes.c_int32) for n in ("delta_pipi_mode", "tau_pipi_mode", "lambda_piPi_mode", "phi6_mode",
                                      "phi7_mode", "delta_PiPi_mode", "lambda_Pipi_mode", "phi1_mode",
                                      "phi3_mode", "restrict_mu_T_ratios")]


def make_config(rc) -> Config:
    c = Config()
    for name, typ in Config._fields_:
        if hasattr(rc, name):
            v = getattr(rc, name)
            if name == "kappa_over_T2":
                v = (ctypes.c_double * 9)(*[float(x) for x in v])
            setattr(c, name, v)
    return c


def build(quiet=True):
    out = subprocess.run(["make", "-C", HERE, "-j8"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(Config), I] + [dp] * 10 + [P]
        L.orc_destroy.argtypes = [P]
        L.orc_initialize.argtypes = [P]
        L.orc_step.argtypes = [P, I]
        L.orc_fo_count.argtypes = [P]
        L.orc_fo_width.argtypes = [P]
        L.orc_fo_rows.argtypes = [P, dp]
        L.orc_fo_rows.restype = None
        L.orc_phase.argtypes = [P, ctypes.c_char_p]
        L.orc_time.restype = D
        L.orc_time.argtypes = [P]
        L.orc_set_time.argtypes = [P, D]
        L.orc_set_initial_viscous.argtypes = [P, I, I]
        L.orc_get.argtypes = [P, ctypes.c_char_p, dp]
        L.orc_set.argtypes = [P, ctypes.c_char_p, dp]
        L.orc_get_int.argtypes = [P, ctypes.c_char_p, ip]
        L.orc_totals.argtypes = [P, dp]
        L.orc_neighbours.restype = ctypes.c_long
        L.orc_neighbours.argtypes = [P, ip, ip, ctypes.c_long]
        L.orc_kernel_W.restype = D
        L.orc_kernel_W.argtypes = [I, D, D]
        L.orc_kernel_gradW.argtypes = [I, dp, D, D, dp]
        L.orc_table_create.restype = P
        L.orc_table_create.argtypes = [ip, dp, dp, dp, dp, dp]
        L.orc_table_destroy.argtypes = [P]
        L.orc_eos_full_thermo.argtypes = [ctypes.POINTER(Config), P, I, dp, dp]
        L.orc_eos_invert_batch.argtypes = [ctypes.POINTER(Config), P, I, ctypes.c_long, dp, dp, dp, ip, ip]
        L.orc_eos_set_thermo.argtypes = [ctypes.POINTER(Config), P, I, dp, dp]
        L.orc_eos_alpha_derivs.argtypes = [ctypes.POINTER(Config), P, I, ctypes.c_long, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class OracleRun:
    """One hydro system on the oracle."""

    def __init__(self, particles, rc, table=None):
        L = lib()
        self.rc = rc
        self.cfg = make_config(rc)
        self.n = particles.n
        arrs = [np.ascontiguousarray(getattr(particles, k), dtype=np.float64)
                for k in ("x", "y", "eta", "e", "rhoB", "rhoS", "rhoQ", "ux", "uy", "ueta")]
        self._keep = arrs
        self.h = L.orc_create(ctypes.byref(self.cfg), self.n, *[_dp(a) for a in arrs],
                              table.h if table is not None else None)

    def __del__(self):
        try:
            lib().orc_destroy(self.h)
        except Exception:
            pass

    def initialize(self) -> int:
        return lib().orc_initialize(self.h)

    def set_initial_viscous(self, trace=None, pi=None):
        """As GpuHydro.set_initial_viscous (before initialize)."""
        if trace is not None:
            self.set("in_bulk", trace)
        if pi is not None:
            for k in range(6):
                self.set(f"in_shv{k}", pi[k])
        lib().orc_set_initial_viscous(self.h, int(trace is not None), int(pi is not None))

    def step(self, n=1) -> int:
        return lib().orc_step(self.h, n)

    def phase(self, name):
        return lib().orc_phase(self.h, name.encode())

    def freeze_out_rows(self):
        """Rows of freeze_out.dat written so far, each (step, particle, fields...)."""
        L = lib()
        k, w = L.orc_fo_count(self.h), L.orc_fo_width(self.h)
        out = np.zeros((k, w))
        if k:
            L.orc_fo_rows(self.h, _dp(out))
        return out

    @property
    def t(self):
        return lib().orc_time(self.h)

    def get(self, name):
        out = np.empty(self.n, dtype=np.float64)
        if lib().orc_get(self.h, name.encode(), _dp(out)) != 0:
            raise KeyError(name)
        return out

    def set(self, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if lib().orc_set(self.h, name.encode(), _dp(v)) != 0:
            raise KeyError(name)

    def get_int(self, name):
        out = np.empty(self.n, dtype=np.int32)
        if lib().orc_get_int(self.h, name.encode(), _ip(out)) != 0:
            raise KeyError(name)
        return out

    def totals(self):
        out = np.zeros(6)
        lib().orc_totals(self.h, _dp(out))
        return dict(zip(("S", "B", "Sq", "Q", "E", "Ez"), out))

    def neighbours(self):
        off = np.zeros(self.n + 1, dtype=np.int32)
        cap = 64 * self.n
        idx = np.zeros(cap, dtype=np.int32)
        m = lib().orc_neighbours(self.h, _ip(off), _ip(idx), cap)
        if m < 0:
            cap = -m
            idx = np.zeros(cap, dtype=np.int32)
            m = lib().orc_neighbours(self.h, _ip(off), _ip(idx), cap)
        return off, idx[:m]


class OracleTable:
    def __init__(self, n, lo, d, fields, conf5, cdiag5):
        self.n = np.asarray(n, dtype=np.int32)
        self.lo = np.asarray(lo, dtype=np.float64)
        self.d = np.asarray(d, dtype=np.float64)
        f = np.ascontiguousarray(fields, dtype=np.float64)
        c5 = np.asarray(conf5, dtype=np.float64)
        d5 = np.asarray(cdiag5, dtype=np.float64)
        self.h = lib().orc_table_create(_ip(self.n), _dp(self.lo), _dp(self.d), _dp(f), _dp(c5), _dp(d5))

    def __del__(self):
        try:
            lib().orc_table_destroy(self.h)
        except Exception:
            pass


def kernel_W(D, r, h):
    return lib().orc_kernel_W(D, r, h)


def kernel_gradW(D, rel, r, h):
    rel = np.ascontiguousarray(rel, dtype=np.float64)
    out = np.zeros(D)
    lib().orc_kernel_gradW(D, _dp(rel), r, h, _dp(out))
    return out


def eos_invert_batch(rc, entropy, targets, seeds=None, table=None):
    """targets: (n, 4) rows (e|s, B, S, Q). Returns tbqs (n,4), th16 (n,16), status, iters."""
    t = np.ascontiguousarray(targets, dtype=np.float64)
    n = t.shape[0]
    x = np.zeros((n, 4)) if seeds is None else np.ascontiguousarray(seeds, dtype=np.float64).copy()
    th = np.zeros((n, 16))
    st = np.zeros(n, dtype=np.int32)
    it = np.zeros(n, dtype=np.int32)
    cfg = make_config(rc)
    lib().orc_eos_invert_batch(ctypes.byref(cfg), table.h if table is not None else None, int(entropy), n,
                               _dp(t), _dp(x), _dp(th), _ip(st), _ip(it))
    return x, th, st, it


THERMO_NAMES = ("T", "muB", "muS", "muQ", "p", "s", "rhoB", "rhoS", "rhoQ", "e", "w", "cs2",
                "dwds", "dwdB", "dwdS", "dwdQ")


def eos_alpha_derivs(rc, chain_index, tbqs, table=None):
    """dalpha_a/ds (columns 0..2) and dalpha_a/drho_b (3 + 3a + b), a, b = B, S, Q,
    at the (T, muB, muQ, muS) rows of tbqs."""
    x = np.ascontiguousarray(tbqs, dtype=np.float64).reshape(-1, 4)
    out = np.zeros((x.shape[0], 12))
    cfg = make_config(rc)
    lib().orc_eos_alpha_derivs(ctypes.byref(cfg), table.h if table is not None else None, int(chain_index),
                               x.shape[0], _dp(x), _dp(out))
    return out
