"""ctypes binding of libccake_gpu.so (the C ABI in include/ccake_gpu.h).

This is the Python-side caller used by the tests and the benchmark. The
library must have been built (``python -m ccake_gb300.build``); loading fails
loudly otherwise -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os

import numpy as np

from . import build as _build

_i32, _i64, _f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


class CcakeConfig(ctypes.Structure):
    _fields_ = [(n, _i32) for n in (
        "dim", "coord", "eos_kind", "using_shear", "using_vorticity", "shear_relax_mode", "zeta_mode",
        "factorized_kernel", "input_as_entropy", "modulate_zeta_with_tanh", "thermo_mode", "precision")] + \
        [(n, _f64) for n in (
            "hT", "hEta", "t0", "dt", "eos_c", "eos_T0", "eos_muB0", "eos_muQ0", "eos_muS0", "eta_over_s",
            "zeta_over_s", "zeta_cs2_A", "zeta_cs2_p", "zeta_peak_T", "zeta_peak_width", "xmin", "ymin",
            "etamin", "freeze_out_T", "skin_frac")] + [("particlization", _i32), ("surface", _i32)] + \
        [(n, _i32) for n in ("using_diffusion", "diffusion_mode", "diffusion_relax_mode", "diffusion_regulator",
                             "critical_scaling_diffusion", "pad2")] + [("kappa_over_T2", _f64 * 9)] + \
        [(n, _f64) for n in ("C_B", "reg_chi0", "reg_e0", "reg_xi0", "reg_rq_max", "crit_T", "crit_muB", "crit_wT",
                             "crit_wmuB")] + \
        [(n, _i32) for n in ("delta_pipi_mode", "tau_pipi_mode", "lambda_piPi_mode", "phi6_mode", "phi7_mode",
                             "delta_PiPi_mode", "lambda_Pipi_mode", "phi1_mode", "phi3_mode", "pad3",
                             "seed_mode", "restrict_mu_T_ratios")]


class ParticlesSoA(ctypes.Structure):
    _fields_ = [("n", _i64)] + [(k, _dp) for k in ("x", "y", "eta", "e_or_s", "rhoB", "rhoS", "rhoQ", "ux",
                                                    "uy", "ueta")]


class PreinvConfig(ctypes.Structure):
    _fields_ = [("exp_lo", _i32 * 4), ("exp_hi", _i32 * 4), ("nodes", _i32), ("reserved", _i32)]


class IcOptions(ctypes.Structure):
    _fields_ = [("input_as_entropy", _i32), ("input_initial_diffusion", _i32), ("baryon", _i32),
                ("strange", _i32), ("electric", _i32), ("reserved", _i32), ("e_cutoff", _f64)]


IC_COLUMNS = ("x", "y", "eta", "e", "rhoB", "rhoS", "rhoQ", "ux", "uy", "ueta", "bulk", "pixx", "pixy", "pixeta",
              "piyy", "piyeta", "pietaeta", "qB0", "qB1", "qB2", "qB3", "qS0", "qS1", "qS2", "qS3", "qQ0", "qQ1",
              "qQ2", "qQ3")


class Totals(ctypes.Structure):
    _fields_ = [(k, _f64) for k in ("S", "B", "Sq", "Q", "E", "Ez")]


STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "EoS inversion failed", 4: "negative entropy",
          5: "buffer too small", 6: "call out of order", 7: "out of device memory", 8: "non-finite state"}


class CcakeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def library_path() -> str:
    return _build.LIB


def lib():
    """Loads libccake_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run `python -m ccake_gb300.build` first")
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.ccake_status_string.restype = ctypes.c_char_p
        L.ccake_status_string.argtypes = [_i32]
        L.ccake_last_error.restype = ctypes.c_char_p
        L.ccake_last_error.argtypes = [P]
        L.ccake_ctx_create.argtypes = [ctypes.POINTER(CcakeConfig), ctypes.POINTER(P)]
        L.ccake_ctx_destroy.argtypes = [P]
        L.ccake_load_particles.argtypes = [P, ctypes.POINTER(ParticlesSoA)]
        L.ccake_preinverted_build.argtypes = [P, ctypes.POINTER(PreinvConfig)]
        L.ccake_preinverted_use.argtypes = [P, _i32]
        L.ccake_preinverted_lookup.argtypes = [P, _i64, _dp, _dp]
        L.ccake_preinverted_copy.argtypes = [P, ctypes.POINTER(_i64), _dp]
        L.ccake_preinverted_lookup_device.argtypes = [P, _i64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.ccake_freeze_out_rows.argtypes = [P, ctypes.POINTER(_i64), ctypes.POINTER(_i32), _dp]
        L.ccake_write_freeze_out.argtypes = [P, ctypes.c_char_p, _f64, _f64, _f64]
        L.ccake_hydro_numbers.argtypes = [P]
        L.ccake_set_initial_diffusion.argtypes = [P, _dp]
        L.ccake_set_initial_viscous.argtypes = [P, _dp, _dp]
        L.ccake_write_system_state.argtypes = [P, ctypes.c_char_p]
        L.ccake_ic_read_ccake.argtypes = [ctypes.c_char_p, ctypes.POINTER(IcOptions), ctypes.POINTER(P)]
        L.ccake_ic_info.argtypes = [P, ctypes.POINTER(_i64), _dp]
        L.ccake_ic_column.argtypes = [P, ctypes.c_char_p, _dp]
        L.ccake_ic_particles.argtypes = [P, ctypes.POINTER(ParticlesSoA)]
        L.ccake_ic_free.argtypes = [P]
        L.ccake_ic_free.restype = None
        for name in ("ccake_initialize", "ccake_build_neighbours", "ccake_smooth_fields", "ccake_update_thermo",
                     "ccake_update_viscosities", "ccake_smooth_gradients", "ccake_time_derivatives"):
            getattr(L, name).argtypes = [P]
        L.ccake_step.argtypes = [P, _i32]
        L.ccake_continue_evolution.argtypes = [P, _f64, ctypes.POINTER(_i32)]
        L.ccake_step_timed.argtypes = [P, _i32, ctypes.POINTER(ctypes.c_float)]
        L.ccake_kernel_launches.argtypes = [P, ctypes.POINTER(_i64)]
        L.ccake_profile_phases.argtypes = [P, _i32, _dp]
        L.ccake_device_bytes.argtypes = [P, ctypes.POINTER(_i64)]
        L.ccake_get_time.argtypes = [P, _dp]
        L.ccake_get_count.argtypes = [P, ctypes.POINTER(_i64)]
        L.ccake_conservation.argtypes = [P, ctypes.POINTER(Totals)]
        L.ccake_copy_out.argtypes = [P, ctypes.c_char_p, _dp]
        L.ccake_copy_out_int.argtypes = [P, ctypes.c_char_p, _ip]
        L.ccake_get_neighbours.argtypes = [P, _ip, _ip, _i64, ctypes.POINTER(_i64)]
        L.ccake_eos_invert_batch.argtypes = [P, _i32, _i64, _dp, _dp, _dp, _ip, _ip]
        L.ccake_eos_invert_batch_ex.argtypes = [P, _i32, _i32, _i64, _dp, _dp, _dp, _ip, _ip]
        L.ccake_eos_invert_device.argtypes = [P, _i32, _i32, _i64, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.ccake_set_eos_table.argtypes = [P, _ip, _dp, _dp, _dp, _dp, _dp]
        L.ccake_eos_thermo_batch.argtypes = [P, _i32, _i64, _dp, _dp]
        L.ccake_set_eos_table_file.argtypes = [P, ctypes.c_char_p, _i32, _dp, _dp]
        L.ccake_eos_table_fallback_scales.argtypes = [_ip, _dp, _dp, _dp, _f64, _dp, _dp]
        L.ccake_sph_kernel.argtypes = [_i32, _f64, _i64, _dp, _dp, _dp]
        _fp = ctypes.POINTER(ctypes.c_float)
        L.ccake_mlp_train.argtypes = [P, _i64, _i32, _i32, ctypes.c_double, ctypes.c_uint64, _dp]
        L.ccake_mlp_get_params.argtypes = [P, _fp, _fp]
        L.ccake_mlp_set_params.argtypes = [P, _fp, _fp]
        L.ccake_mlp_forward.argtypes = [P, _i64, _fp, _fp]
        L.ccake_mlp_gradient.argtypes = [P, _i64, _fp, _fp, _fp, _dp]
        _lib = L
    return _lib


def make_config(rc) -> CcakeConfig:
    c = CcakeConfig()
    for name, _ in CcakeConfig._fields_:
        if hasattr(rc, name):
            v = getattr(rc, name)
            if name == "kappa_over_T2":
                v = (_f64 * 9)(*[float(x) for x in v])
            setattr(c, name, v)
    return c


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def sph_kernel(dim, h, r2):
    """(W, fg) of the cubic spline at squared distances r2, evaluated on the
    GPU by the device function of the FP64 pair loops (ccake_sph_kernel):
    W = SPHkernel<dim>::kernel(sqrt(r2), h), grad W = fg * rel."""
    r2 = np.ascontiguousarray(r2, dtype=np.float64)
    w, fg = np.zeros_like(r2), np.zeros_like(r2)
    code = lib().ccake_sph_kernel(int(dim), float(h), r2.size, _d(r2), _d(w), _d(fg))
    if code:
        raise CcakeError(code, "sph_kernel")
    return w, fg


def table_fallback_scales(n, lo, d, fields, freeze_out_T):
    """(conf5, cdiag5) of the analytic fallbacks matched to a table as the
    reference does (ccake_eos_table_fallback_scales)."""
    n = np.ascontiguousarray(n, dtype=np.int32)
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    f = np.ascontiguousarray(fields, dtype=np.float64)
    c5, d5 = np.zeros(5), np.zeros(5)
    code = lib().ccake_eos_table_fallback_scales(_i(n), _d(lo), _d(d), _d(f), float(freeze_out_T), _d(c5), _d(d5))
    if code:
        raise CcakeError(code, "eos_table_fallback_scales")
    return c5, d5


class GpuHydro:
    """One event resident on the GPU, driven through the C ABI."""

    def __init__(self, rc):
        L = lib()
        self.rc = rc
        self.cfg = make_config(rc)
        self.h = ctypes.c_void_p()
        self._check(L.ccake_ctx_create(ctypes.byref(self.cfg), ctypes.byref(self.h)), "create")
        self.n = 0

    def _check(self, code, what):
        if code != 0:
            msg = lib().ccake_last_error(self.h).decode() if self.h else ""
            raise CcakeError(code, f"{what}: {msg}")

    def close(self):
        if self.h:
            lib().ccake_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, particles):
        arrs = {k: np.ascontiguousarray(getattr(particles, k), dtype=np.float64)
                for k in ("x", "y", "eta", "e", "rhoB", "rhoS", "rhoQ", "ux", "uy", "ueta")}
        self._keep = arrs
        soa = ParticlesSoA(particles.n, _d(arrs["x"]), _d(arrs["y"]), _d(arrs["eta"]), _d(arrs["e"]),
                           _d(arrs["rhoB"]), _d(arrs["rhoS"]), _d(arrs["rhoQ"]), _d(arrs["ux"]),
                           _d(arrs["uy"]), _d(arrs["ueta"]))
        self._check(lib().ccake_load_particles(self.h, ctypes.byref(soa)), "load")
        self.n = particles.n

    def set_initial_viscous(self, trace=None, pi=None):
        """Initial bulk (trace input of bulk_from_trace, n) and/or shear (pi[6, n]:
        xx xy xeta yy yeta etaeta) of the loaded particles; between load and initialize."""
        tr = None if trace is None else np.ascontiguousarray(trace, dtype=np.float64)
        pv = None if pi is None else np.ascontiguousarray(pi, dtype=np.float64)
        if tr is not None and tr.shape != (self.n,):
            raise ValueError("trace must have shape (n,)")
        if pv is not None and pv.shape != (6, self.n):
            raise ValueError("pi must have shape (6, n)")
        self._keep_visc = (tr, pv)
        self._check(lib().ccake_set_initial_viscous(self.h, None if tr is None else tr.ctypes.data_as(_dp),
                                                    None if pv is None else pv.ctypes.data_as(_dp)),
                    "set_initial_viscous")

    def set_initial_diffusion(self, q):
        """Initial diffusion currents, q[4 c + mu, i] = q^mu of charge c (B, S,
        Q) of particle i (the spatial q^i are used); between load and initialize."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.shape != (12, self.n):
            raise ValueError("q must have shape (12, n)")
        self._check(lib().ccake_set_initial_diffusion(self.h, q.ctypes.data_as(_dp)), "set_initial_diffusion")

    def initialize(self):
        self._check(lib().ccake_initialize(self.h), "initialize")

    def step(self, n=1):
        self._check(lib().ccake_step(self.h, int(n)), "step")

    def preinverted_build(self, exp_lo=(-3, -3, -3, -3), exp_hi=(1, 0, 0, 0), nodes=20):
        """Pre-inverted (s, rho) -> thermodynamics tables from this context's
        EoS (ccake_preinverted_build; defaults: the reference generator's)."""
        c = PreinvConfig((_i32 * 4)(*exp_lo), (_i32 * 4)(*exp_hi), int(nodes), 0)
        self._check(lib().ccake_preinverted_build(self.h, ctypes.byref(c)), "preinverted_build")

    def preinverted_use(self, on=True):
        self._check(lib().ccake_preinverted_use(self.h, 1 if on else 0), "preinverted_use")

    def preinverted_lookup(self, sBSQ):
        """(n, 4) densities -> (n, 11): T, muB, muQ, muS, e, p, cs2, dwds, dwdB, dwdQ, dwdS."""
        a = np.ascontiguousarray(sBSQ, dtype=np.float64).reshape(-1, 4)
        out = np.zeros((a.shape[0], 11))
        self._check(lib().ccake_preinverted_lookup(self.h, a.shape[0], _d(a), _d(out)), "preinverted_lookup")
        return out

    def preinverted_lookup_device(self, n, in4_ptr, out11_ptr, stream_ptr=None):
        """ccake_preinverted_lookup_device on device pointers (ints), asynchronous."""
        self._check(lib().ccake_preinverted_lookup_device(self.h, int(n), in4_ptr, out11_ptr, stream_ptr),
                    "preinverted_lookup_device")

    def preinverted_values(self):
        n = _i64()
        self._check(lib().ccake_preinverted_copy(self.h, ctypes.byref(n), None), "preinverted_copy")
        out = np.zeros((n.value, 11))
        self._check(lib().ccake_preinverted_copy(self.h, ctypes.byref(n), _d(out)), "preinverted_copy")
        return out

    def freeze_out_rows(self):
        """Hypersurface rows so far (cfg.surface): (count, 2 + fields), each
        step, particle, then the freeze_out.dat fields."""
        k, w = _i64(), _i32()
        self._check(lib().ccake_freeze_out_rows(self.h, ctypes.byref(k), ctypes.byref(w), None), "freeze_out_rows")
        out = np.zeros((k.value, w.value))
        if k.value:
            self._check(lib().ccake_freeze_out_rows(self.h, ctypes.byref(k), ctypes.byref(w), _d(out)),
                        "freeze_out_rows")
        return out

    def write_freeze_out(self, path, B=0.0, S=0.0, Q=0.0):
        """freeze_out.dat with the header "# B S Q"."""
        self._check(lib().ccake_write_freeze_out(self.h, os.fsencode(path), float(B), float(S), float(Q)),
                    "write_freeze_out")

    def hydro_numbers(self):
        """theta, sigma^{ij}, Knudsen and inverse Reynolds numbers and the
        transport coefficients of the last derivative evaluation, into the
        fields of get() (ccake_hydro_numbers)."""
        self._check(lib().ccake_hydro_numbers(self.h), "hydro_numbers")

    def write_system_state(self, path):
        """The reference's system_state_<n>.dat text output at path."""
        self._check(lib().ccake_write_system_state(self.h, os.fsencode(path)), "write_system_state")

    def continue_evolution(self, max_tau):
        """The reference's stop rule: False once every particle froze out (particlization) or t > max_tau."""
        k = _i32()
        self._check(lib().ccake_continue_evolution(self.h, float(max_tau), ctypes.byref(k)), "continue_evolution")
        return bool(k.value)

    def step_timed(self, n):
        """Advances n steps; returns the device time (ms) measured on the library's stream."""
        ms = ctypes.c_float()
        self._check(lib().ccake_step_timed(self.h, int(n), ctypes.byref(ms)), "step_timed")
        return float(ms.value)

    def kernel_launches(self):
        """Kernels launched by step / step_timed on this context so far (graph kernel nodes x launches)."""
        v = ctypes.c_int64()
        self._check(lib().ccake_kernel_launches(self.h, ctypes.byref(v)), "kernel_launches")
        return int(v.value)

    def profile_phases(self, n):
        """Average device ms per launch: (cell-list kernels, pass A, pass B)."""
        out = np.zeros(3)
        self._check(lib().ccake_profile_phases(self.h, int(n), _d(out)), "profile_phases")
        return out

    def device_bytes(self):
        v = ctypes.c_int64()
        self._check(lib().ccake_device_bytes(self.h, ctypes.byref(v)), "device_bytes")
        return int(v.value)

    def phase(self, name):
        self._check(getattr(lib(), "ccake_" + name)(self.h), name)

    @property
    def t(self):
        v = ctypes.c_double()
        self._check(lib().ccake_get_time(self.h, ctypes.byref(v)), "time")
        return v.value

    def get(self, name):
        out = np.empty(self.n, dtype=np.float64)
        self._check(lib().ccake_copy_out(self.h, name.encode(), _d(out)), f"copy_out {name}")
        return out

    def get_int(self, name):
        out = np.empty(self.n, dtype=np.int32)
        self._check(lib().ccake_copy_out_int(self.h, name.encode(), _i(out)), f"copy_out_int {name}")
        return out

    def totals(self):
        t = Totals()
        self._check(lib().ccake_conservation(self.h, ctypes.byref(t)), "conservation")
        return {k: getattr(t, k) for k, _ in Totals._fields_}

    def neighbours(self):
        off = np.zeros(self.n + 1, dtype=np.int32)
        cnt = ctypes.c_int64()
        code = lib().ccake_get_neighbours(self.h, _i(off), None, 0, ctypes.byref(cnt))
        if code not in (0, 5):
            self._check(code, "neighbours")
        idx = np.zeros(max(cnt.value, 1), dtype=np.int32)
        self._check(lib().ccake_get_neighbours(self.h, _i(off), _i(idx), cnt.value, ctypes.byref(cnt)),
                    "neighbours")
        return off, idx[:cnt.value]

    def set_eos_table(self, n, lo, d, fields, conf5=None, cdiag5=None):
        """Uploads a tabulated EoS (eos_kind 2); see ccake_set_eos_table. Fallback
        scales left as None are matched to the table as the reference does."""
        n = np.ascontiguousarray(n, dtype=np.int32)
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        d = np.ascontiguousarray(d, dtype=np.float64)
        f = np.ascontiguousarray(fields, dtype=np.float64)
        c5 = None if conf5 is None else np.ascontiguousarray(conf5, dtype=np.float64)
        d5 = None if cdiag5 is None else np.ascontiguousarray(cdiag5, dtype=np.float64)
        self._check(lib().ccake_set_eos_table(self.h, _i(n), _d(lo), _d(d), _d(f), _d(c5), _d(d5)), "set_eos_table")

    def set_eos_table_file(self, path, normalize_by_T, conf5=None, cdiag5=None):
        """Loads a thermo.dat table (the reference's text format); see ccake_set_eos_table_file."""
        c5 = None if conf5 is None else np.ascontiguousarray(conf5, dtype=np.float64)
        d5 = None if cdiag5 is None else np.ascontiguousarray(cdiag5, dtype=np.float64)
        self._check(lib().ccake_set_eos_table_file(self.h, str(path).encode(), int(bool(normalize_by_T)), _d(c5),
                                                   _d(d5)), "set_eos_table_file")

    def eos_thermo(self, chain_index, tbqs):
        """17 model fields at rows (T, muB, muQ, muS) for EoS chain index chain_index."""
        x = np.ascontiguousarray(tbqs, dtype=np.float64)
        out = np.zeros((x.shape[0], 17))
        self._check(lib().ccake_eos_thermo_batch(self.h, int(chain_index), x.shape[0], _d(x), _d(out)),
                    "eos_thermo_batch")
        return out

    def eos_invert_device(self, entropy, seed_mode, n, in4_ptr, tbqs_ptr, th16_ptr, status_ptr, iters_ptr,
                          stream_ptr=None):
        """ccake_eos_invert_device on device pointers (ints); asynchronous on the stream."""
        self._check(lib().ccake_eos_invert_device(self.h, int(entropy), int(seed_mode), int(n), in4_ptr, tbqs_ptr,
                                                  th16_ptr, status_ptr, iters_ptr, stream_ptr),
                    "eos_invert_device")

    # -- learned Newton seed -------------------------------------------------------
    def mlp_train(self, n_samples=5_000_000, epochs=20, batch=32768, lr=3e-3, seed=1):
        """Trains the seed network on table samples; returns the last epoch's MSE (standardised)."""
        mse = ctypes.c_double()
        self._check(lib().ccake_mlp_train(self.h, int(n_samples), int(epochs), int(batch), float(lr), int(seed),
                                          ctypes.byref(mse)), "mlp_train")
        return float(mse.value)

    def mlp_params(self):
        prm = np.zeros(8900, dtype=np.float32)
        norm = np.zeros(16, dtype=np.float32)
        self._check(lib().ccake_mlp_get_params(self.h, _f(prm), _f(norm)), "mlp_get_params")
        return prm, norm

    def mlp_set_params(self, prm, norm):
        prm = np.ascontiguousarray(prm, dtype=np.float32)
        norm = np.ascontiguousarray(norm, dtype=np.float32)
        self._check(lib().ccake_mlp_set_params(self.h, _f(prm), _f(norm)), "mlp_set_params")

    def mlp_forward(self, feat):
        f = np.ascontiguousarray(feat, dtype=np.float32)
        out = np.zeros_like(f)
        self._check(lib().ccake_mlp_forward(self.h, f.shape[0], _f(f), _f(out)), "mlp_forward")
        return out

    def mlp_gradient(self, feat, tgt):
        f = np.ascontiguousarray(feat, dtype=np.float32)
        t = np.ascontiguousarray(tgt, dtype=np.float32)
        g = np.zeros(8900, dtype=np.float32)
        sse = ctypes.c_double()
        self._check(lib().ccake_mlp_gradient(self.h, f.shape[0], _f(f), _f(t), _f(g), ctypes.byref(sse)),
                    "mlp_gradient")
        return g, float(sse.value)

    def eos_invert(self, entropy, targets, seeds, seed_mode=0):
        """Batch inversion; seed_mode 0 reference seed chain, 1 analytic exact inverse first."""
        t = np.ascontiguousarray(targets, dtype=np.float64)
        x = np.ascontiguousarray(seeds, dtype=np.float64).copy()
        n = t.shape[0]
        th = np.zeros((n, 16))
        st = np.zeros(n, dtype=np.int32)
        it = np.zeros(n, dtype=np.int32)
        self._check(lib().ccake_eos_invert_batch_ex(self.h, int(entropy), int(seed_mode), n, _d(t), _d(x), _d(th),
                                                    _i(st), _i(it)), "eos_invert_batch")
        return x, th, st, it


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", _i64), ("max_active", _i32), ("steps_per_launch", _i32)]


class EventResult(ctypes.Structure):
    _fields_ = [("ticket", _i64), ("particles", _i64), ("state", _i32), ("status", _i32), ("steps", _i32),
                ("frozen", _i32), ("tau", _f64), ("queue_s", _f64), ("latency_s", _f64), ("device_bytes", _i64),
                ("grouped", _i32), ("reserved", _i32)]


def estimate_device_bytes(rc, n):
    """Device bytes the event server reserves for an event of n particles (ccake_estimate_device_bytes)."""
    cfg = make_config(rc)
    v = _i64()
    lib().ccake_estimate_device_bytes.argtypes = [ctypes.POINTER(CcakeConfig), _i64, ctypes.POINTER(_i64)]
    code = lib().ccake_estimate_device_bytes(ctypes.byref(cfg), int(n), ctypes.byref(v))
    if code:
        raise CcakeError(code, "estimate_device_bytes")
    return int(v.value)


class Server:
    """ccake_server_*: continuous batching of independent events on one GPU."""

    STATES = {0: "queued", 1: "running", 2: "done", 3: "failed"}

    def __init__(self, hbm_budget_bytes=0, max_active=0, steps_per_launch=0):
        L = lib()
        P = ctypes.c_void_p
        L.ccake_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(P)]
        L.ccake_server_destroy.argtypes = [P]
        L.ccake_server_submit.argtypes = [P, ctypes.POINTER(CcakeConfig), ctypes.POINTER(ParticlesSoA), _f64,
                                          ctypes.POINTER(_i64)]
        L.ccake_server_poll.argtypes = [P, _i64, ctypes.POINTER(EventResult)]
        L.ccake_server_wait_all.argtypes = [P]
        L.ccake_server_copy_out.argtypes = [P, _i64, ctypes.c_char_p, _dp]
        L.ccake_server_release.argtypes = [P, _i64]
        cfg = ServerConfig(int(hbm_budget_bytes), int(max_active), int(steps_per_launch))
        self.h = P()
        code = L.ccake_server_create(ctypes.byref(cfg), ctypes.byref(self.h))
        if code:
            raise CcakeError(code, "server_create")
        self._n = {}

    def submit(self, particles, rc, tau_max):
        cfg = make_config(rc)
        arrs = {k: np.ascontiguousarray(getattr(particles, k), dtype=np.float64)
                for k in ("x", "y", "eta", "e", "rhoB", "rhoS", "rhoQ", "ux", "uy", "ueta")}
        soa = ParticlesSoA(particles.n, _d(arrs["x"]), _d(arrs["y"]), _d(arrs["eta"]), _d(arrs["e"]),
                           _d(arrs["rhoB"]), _d(arrs["rhoS"]), _d(arrs["rhoQ"]), _d(arrs["ux"]),
                           _d(arrs["uy"]), _d(arrs["ueta"]))
        t = _i64()
        code = lib().ccake_server_submit(self.h, ctypes.byref(cfg), ctypes.byref(soa), float(tau_max),
                                         ctypes.byref(t))
        if code:
            raise CcakeError(code, "server_submit")
        self._n[t.value] = particles.n
        return t.value

    def poll(self, ticket):
        r = EventResult()
        code = lib().ccake_server_poll(self.h, int(ticket), ctypes.byref(r))
        if code:
            raise CcakeError(code, "server_poll")
        d = {k: getattr(r, k) for k, _ in EventResult._fields_}
        d["state"] = self.STATES[d["state"]]
        return d

    def wait_all(self):
        lib().ccake_server_wait_all(self.h)

    def get(self, ticket, field):
        out = np.empty(self._n[ticket], dtype=np.float64)
        code = lib().ccake_server_copy_out(self.h, int(ticket), field.encode(), _d(out))
        if code:
            raise CcakeError(code, f"server_copy_out {field}")
        return out

    def release(self, ticket):
        lib().ccake_server_release(self.h, int(ticket))
        self._n.pop(ticket, None)

    def close(self):
        if getattr(self, "h", None):
            lib().ccake_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def exported_symbols():
    """Names declared in include/ccake_gpu.h."""
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ccake_gpu.h")
    src = open(hdr).read()
    return sorted(set(re.findall(r"\b(ccake_[a-z_0-9]+)\s*\(", src)))


def read_ccake_ic(path, input_as_entropy=0, input_initial_diffusion=0, charges=(1, 1, 1), e_cutoff=0.0):
    """Reads a "ccake" initial-condition file through the library
    (ccake_ic_read_ccake, the rules of src/BSQHydro.cpp:206-425).

    Returns (particles, columns, grid): an ics.Particles for GpuHydro.load,
    every column by name (internal units: e, bulk and pi^{ij} divided by
    hbar c), and (dx, dy, deta, xmin, ymin, etamin) from the header."""
    from . import ics
    L = lib()
    opt = IcOptions(int(input_as_entropy), int(input_initial_diffusion), int(charges[0]), int(charges[1]),
                    int(charges[2]), 0, float(e_cutoff))
    h = ctypes.c_void_p()
    code = L.ccake_ic_read_ccake(os.fsencode(path), ctypes.byref(opt), ctypes.byref(h))
    if code != 0:
        raise CcakeError(code, f"read_ccake_ic {path}: {L.ccake_status_string(code).decode()}")
    try:
        n = _i64()
        grid = np.zeros(6)
        L.ccake_ic_info(h, ctypes.byref(n), _d(grid))
        cols = {}
        for name in IC_COLUMNS:
            a = np.zeros(n.value)
            code = L.ccake_ic_column(h, name.encode(), _d(a))
            if code != 0:
                raise CcakeError(code, f"ccake_ic_column {name}")
            cols[name] = a
    finally:
        L.ccake_ic_free(h)
    p = ics.Particles(x=cols["x"], y=cols["y"], eta=cols["eta"], e=cols["e"], rhoB=cols["rhoB"],
                      rhoS=cols["rhoS"], rhoQ=cols["rhoQ"], ux=cols["ux"], uy=cols["uy"], ueta=cols["ueta"])
    return p, cols, tuple(float(v) for v in grid)
