"""Benchmark of the SPH hot path: particle-steps/s on the viscous 2+1-D BSQ event.

Workload (one GPU): 400 x 400 = 160,000 particles, dx = 0.05 fm, h = 0.1 fm,
30 Gaussian hot spots (seeded), conformal-diagonal EoS with B and Q charge,
eta/s = 0.08 with tau_pi = 5 eta/w, midpoint RK2 at dt = 0.001 fm/c, plain
FP64. One "step" is one RK2 step (two derivative evaluations) of every
particle. Synthetic data generated in memory.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs under torchrun: every rank advances its own independent event
(replicas; the path has no cross-event exchange), the slowest rank's time is
reported and value counts the particles of all ranks.

--impl reference times the reference algorithm on the host cores: the
reference itself (Kokkos/Cabana/GSL/HDF5/yaml-cpp) cannot be built here, so
its CPU restatement in oracle/ (C++17/OpenMP, all host threads) is timed.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (plain FP64, viscous BSQ 2+1-D hot-spot event)"
UNIT = "particle-steps/s"


def workload(n_side=400):
    from ccake_gb300 import ics
    return ics.hotspots_2d(n_side=n_side)


def config_dict(n):
    """The workload, identical in both arms."""
    return {"workload": "viscous 2+1-D BSQ, 30 hot spots, 400x400 lattice (160k particles), dx=0.05 fm, h=0.1 fm, "
                        "conformal-diagonal EoS, eta/s=0.08, RK2 dt=0.001 fm/c",
            "particles_per_gpu": n, "precision": "fp64",
            "l2": "resident event state larger than the 129 MB L2 (no flush)"}


def cpu_model():
    """The host CPU's model name (lscpu), for the CPU-baseline lines."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


# -- clocks during the timed region ----------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self, gpu_index=0):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                if int(f[0]) != gpu_index:
                    continue
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def fp64_peak_tflops():
    """FP64 DGEMM throughput of this GPU (torch/cuBLAS, 8192^3), the FP64 pipe ceiling."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def read_traffic(kernel):
    """DRAM bytes per launch from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def read_mixed_traffic():
    """DRAM bytes per launch of the mixed-form kernels from the committed ncu summary."""
    out = {}
    for k in ("passA_mixed", "thermo_fast", "thermo_mixed", "passB_mixed", "eom_mixed"):
        v = read_traffic(k)
        if v is not None:
            out[k] = v
    return out


# -- the reference arm ---------------------------------------------------------------------------
def _oracle():
    import ctypes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as O
    O.build()
    O.lib().orc_set_threads.argtypes = [ctypes.c_int]
    return O


def cpu_reference(p, rc, steps, warmup=1, threads=0, keep=False):
    """Times the oracle (CPU restatement of the reference): `warmup` untimed
    RK2 steps, then `steps` timed ones, on `threads` OpenMP threads (0: all
    host cores). Returns (particle-steps/s, seconds, the run if keep)."""
    O = _oracle()
    O.lib().orc_set_threads(int(threads))
    r = O.OracleRun(p, rc)
    if r.initialize() != 0:
        raise RuntimeError("oracle initialisation failed")
    if warmup:
        r.step(warmup)
    t0 = time.perf_counter()
    r.step(steps)
    dt = time.perf_counter() - t0
    O.lib().orc_set_threads(0)
    return p.n * steps / dt, dt, (r if keep else None)


def run_reference(args, world, rank):
    if rank != 0:
        return
    p, rc = workload()
    value, dt, _ = cpu_reference(p, rc, args.steps, warmup=args.warmup)
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(p.n), "host": "cpu",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "cpu_model": cpu_model(),
                             "sample": f"{args.warmup} warm-up then {args.steps} timed RK2 steps of all {p.n} "
                                       f"particles, OMP threads={cores}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's Kokkos/Cabana build needs dependencies absent here; its CPU restatement "
                    "(oracle/, same algorithms) is timed"}
    print(json.dumps(line))


# -- our arm ---------------------------------------------------------------------------------
def run_ours(args, world, rank):
    import torch
    from ccake_gb300 import api, build

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    build.build()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    p, rc = workload()
    n = p.n
    gpu = api.GpuHydro(rc)
    gpu.load(p)
    gpu.initialize()
    for _ in range(args.warmup):
        gpu.step(1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler()
    if rank == 0:
        clocks.start()
        time.sleep(0.3)
    launches0 = gpu.kernel_launches()
    ms = gpu.step_timed(args.steps)
    launches = gpu.kernel_launches() - launches0
    torch.cuda.synchronize()
    clk = clocks.stop(local) if rank == 0 else None
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if dist:
        dist.barrier()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * n * args.steps / (ms_max * 1e-3)
    # per-kernel device times (events on the library's stream), kernel by kernel
    prof = gpu.profile_phases(max(2, min(10, args.steps)))
    # end to end through the C ABI with host buffers (upload, initialise, K steps, download)
    e2e = run_e2e(p, rc, args.steps)
    mixed = run_mixed(p, rc, args, world, dist)
    if dist:
        dist.destroy_process_group()
    if rank != 0:
        return
    hbm_peak, peak_kind = measured_peaks()
    # algorithmic bytes and FP64 operations per launch from the committed
    # traffic model (ccake_gb300/traffic_model.py, config C2)
    from ccake_gb300 import traffic_model as TM
    alg = {"cells": TM.bytes_per_launch("C2", "binning", n), "passA": TM.bytes_per_launch("C2", "passA", n),
           "passB": TM.bytes_per_launch("C2", "passB", n)}
    flops = {"cells": 0.0, "passA": TM.flops_per_launch("C2", "passA", n),
             "passB": TM.flops_per_launch("C2", "passB", n)}
    names = ["cells", "passA", "passB"]
    dom = int(np.argmax(prof))
    kname = names[dom]
    fp64 = None
    try:
        fp64 = fp64_peak_tflops()
    except Exception:
        pass
    fp64_ach = flops[kname] / (prof[dom] * 1e-3) / 1e12
    hbm_ach = alg[kname] / (prof[dom] * 1e-3) / 1e9
    traffic = read_traffic(kname)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(n),
        "parallelism": f"replicas{world}", "device_bytes": gpu.device_bytes(),
        "clocks": clk,
        "gpu_launches": launches,
        "e2e": e2e,
        "mixed": mixed,
        # the dominant FP64 pass is bound by the FP64 pipe (ncu: the FP64 pipe
        # is the busiest unit, DRAM under 3 %); its roofline is the FP64 peak,
        # with the HBM fraction of the algorithmic bytes beside it
        "roofline": {"bound": "fp64", "kernel": kname, "achieved": fp64_ach, "peak": fp64, "unit": "TFLOP/s",
                     "frac": (fp64_ach / fp64) if fp64 else None,
                     "peak_kind": "measured on this GPU in the same process: cuBLAS DGEMM 8192^3 (no FP64 entry "
                                  "in MEASURED_PEAKS.json)",
                     "traffic": traffic, "avg_launch_ms": prof[dom],
                     "flops_per_launch": flops[kname],
                     "phase_ms": dict(zip(names, [float(x) for x in prof])),
                     "hbm": {"achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_ach / hbm_peak,
                             "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg[kname]}},
    }
    if not args.no_cpu:
        # the CPU baseline leg: the oracle on the host cores, 100 RK2 steps of
        # the same event; its final state is also the reference of the
        # accuracy block (FP64 and mixed GPU forms after the same 100 steps)
        O = _oracle()
        cv, cdt, orc = cpu_reference(p, rc, ACC_STEPS, warmup=0, keep=True)
        c1, _, _ = cpu_reference(p, rc, 1, warmup=0, threads=1)
        line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "cpu_model": cpu_model(),
                                "sample": f"{ACC_STEPS} RK2 steps of the same 160k-particle event from its initial "
                                          f"state on the host (oracle/, OpenMP, {os.cpu_count()} threads)",
                                "one_thread": {"value": c1, "unit": UNIT, "sample": "1 RK2 step, 1 thread"}}
        mixed["accuracy"] = accuracy_vs_oracle(p, rc, orc, O)
        mixed["error_reference"] = "oracle"
    print(json.dumps(line))


ACC_STEPS = 100


def accuracy_vs_oracle(p, rc, orc, O):
    """Per-particle error of the FP64 and mixed GPU forms after ACC_STEPS
    RK2 steps against the oracle's state after the same steps (plain
    relative error of e and the densities; velocities against their range),
    on the 160k event and on the same event with strangeness (rhoS = 0.2
    rhoB cos x), so that all four densities are checked."""
    import dataclasses
    from ccake_gb300 import api, ics
    fields = ("e", "rhoB", "rhoS", "rhoQ", "s", "T")

    def gpu_state(pp, rcc, prec):
        h = api.GpuHydro(dataclasses.replace(rcc, precision=prec))
        h.load(pp)
        h.initialize()
        h.step(ACC_STEPS)
        out = {f: h.get(f) for f in fields + ("u0", "u1")}
        out["totals"] = h.totals()
        h.close()
        return out

    def errors(g, o_get, o_tot):
        err = {}
        for f in fields:
            b = o_get(f)
            big = np.abs(b) >= 1e-3 * np.max(np.abs(b)) if np.any(b) else np.zeros(b.shape, bool)
            if big.any():
                err[f] = float(np.max(np.abs(g[f][big] - b[big]) / np.abs(b[big])))
        for f in ("u0", "u1"):
            b = o_get(f)
            err[f + "_of_range"] = float(np.max(np.abs(g[f] - b)) / (np.max(np.abs(b)) + 1e-300))
        tot = {k: float(abs(g["totals"][k] - o_tot[k]) / (abs(o_tot[k]) + 1e-300)) for k in ("S", "B", "Q", "E")}
        return {"max_rel_err": err, "totals_rel_diff": tot}

    out = {"steps": ACC_STEPS}
    o_tot = orc.totals()
    for prec, name in ((0, "fp64"), (1, "mixed")):
        out[name] = errors(gpu_state(p, rc, prec), orc.get, o_tot)
    ps, rcs = ics.hotspots_2d(n_side=400, rhoS_frac=0.2)
    o2 = O.OracleRun(ps, rcs)
    o2.initialize()
    o2.step(ACC_STEPS)
    o2_tot = o2.totals()
    out["with_strangeness"] = {name: errors(gpu_state(ps, rcs, prec), o2.get, o2_tot)
                               for prec, name in ((0, "fp64"), (1, "mixed"))}
    out["note"] = ("max over particles of |gpu - oracle| / |oracle| where |oracle| >= 1e-3 of the field's "
                   "largest magnitude; the mixed form's bar is 1e-5 in e and rhoB, rhoS, rhoQ")
    return out


def run_mixed(p, rc, args, world, dist):
    """The mixed-precision form (FP32 compensated pair sums, FP32 EoM, FP64
    EoS/state) on the same event: throughput and per-kernel times. Its error
    against the oracle is added by the CPU-baseline leg."""
    import dataclasses
    import torch
    from ccake_gb300 import api
    mrc = dataclasses.replace(rc, precision=1)
    g = api.GpuHydro(mrc)
    g.load(p)
    g.initialize()
    for _ in range(args.warmup):
        g.step(1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    l0 = g.kernel_launches()
    ms = g.step_timed(args.steps)
    launches = g.kernel_launches() - l0
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    prof = g.profile_phases(max(2, min(10, args.steps)))
    g.close()
    n = p.n
    from ccake_gb300 import traffic_model as TM
    hbm_peak, peak_kind = measured_peaks()
    names = ["cells", "passA", "passB"]
    dom = int(np.argmax(prof))
    alg = TM.bytes_per_launch("C2", {"cells": "binning"}.get(names[dom], names[dom]), n)
    ach = alg / (prof[dom] * 1e-3) / 1e9
    return {"value": world * n * args.steps / (ms_max * 1e-3), "unit": UNIT, "ms_per_step": ms_max / args.steps,
            "phase_ms": dict(zip(names, [float(x) for x in prof])),
            "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                         "frac": ach / hbm_peak, "peak_kind": peak_kind,
                         "traffic_per_substep_bytes": sum(v for k, v in read_mixed_traffic().items()),
                         "note": "pass A = smoothing + EoS kernels, pass B = gradient + EoM kernels"},
            "gpu_launches": launches,
            "error_reference": "none (run without the CPU leg)",
            "what": "FP32 pair loops with Kahan sums and (hi, lo) float positions, FP32 EoM; FP64 EoS Newton, "
                    "state, RK2 update and totals"}


def run_e2e(p, rc, steps):
    """Same metric through the C ABI with host buffers: load (H2D), initialise,
    K steps, copy the evolved state back (D2H), all inside the timed region."""
    from ccake_gb300 import api
    out_fields = ["x", "y", "u0", "u1", "ext_s", "ext_bulk", "ext_shv0", "ext_shv1", "ext_shv3", "T", "e"]
    t0 = time.perf_counter()
    g = api.GpuHydro(rc)
    g.load(p)
    g.initialize()
    g.step(steps)
    outs = [g.get(f) for f in out_fields]
    dt = time.perf_counter() - t0
    g.close()
    n = p.n
    h2d = 10 * 8 * n
    d2h = sum(o.nbytes for o in outs)
    return {"value": n * steps / dt, "unit": UNIT, "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": d2h / steps, "wall_s": dt,
            "what": "ccake_load_particles + ccake_initialize + ccake_step(K) + ccake_copy_out of 11 fields"}


def run_eos_table(args):
    """EoS-inversion stress test: the synthetic 4-D table (151 x 41^3 nodes,
    FP64), 2M states uniform in its (T, mu) box mapped forward to
    (e, rhoB, rhoS, rhoQ) through the table and inverted on the GPU (energy
    mode, the reference's seed chain and cs2 guards). Reports inversions/s,
    Newton iterations, the rate of rows solved by a fallback model or not at
    all, and the error of table-solved rows against the drawn states."""
    import torch
    from ccake_gb300 import api, build, eos_table, ics
    build.build()
    n_rows = args.eos_rows
    n, lo, d, fields = eos_table.synthetic_table()
    rc = ics.RunConfig(eos_kind=2, thermo_mode=1)
    # the analytic fallbacks (tanh-conformal, conformal, conformal-diagonal)
    # matched to the table as the reference does
    conf5, cdiag5 = api.table_fallback_scales(n, lo, d, fields, rc.freeze_out_T)
    g = api.GpuHydro(rc)
    g.set_eos_table(n, lo, d, fields, conf5, cdiag5)
    x_true = eos_table.sample_states(n_rows, seed=1)
    fw = g.eos_thermo(0, x_true)
    tgt = np.ascontiguousarray(np.column_stack([fw[:, 5], fw[:, 2], fw[:, 3], fw[:, 4]]))
    dev = torch.device("cuda")
    d_in = torch.from_numpy(tgt).to(dev)
    seed0 = torch.tensor([580 / 197.3269804, 0, 0, 0], dtype=torch.float64, device=dev).repeat(n_rows, 1)
    d_x = seed0.clone()
    d_th = torch.empty((n_rows, 16), dtype=torch.float64, device=dev)
    d_st = torch.empty(n_rows, dtype=torch.int32, device=dev)
    d_it = torch.empty(n_rows, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()

    def timed(seed_mode):
        def run_once():
            d_x.copy_(seed0)
            g.eos_invert_device(0, seed_mode, n_rows, d_in.data_ptr(), d_x.data_ptr(), d_th.data_ptr(),
                                d_st.data_ptr(), d_it.data_ptr(), stream.cuda_stream)

        for _ in range(max(1, args.warmup)):
            run_once()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            run_once()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps, d_x.cpu().numpy(), d_st.cpu().numpy(), d_it.cpu().numpy()

    # learned seed: the seed network trained on 5M table samples (BF16 tensor cores)
    t0 = time.perf_counter()
    mse = g.mlp_train(n_samples=5_000_000, epochs=20, batch=32768, lr=3e-3, seed=2)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    msl, xl, stl, itl = timed(2)
    ms, x, st, it = timed(0)
    tab = st == 0
    hb = eos_table.HBARC
    # states where the EoS is thermodynamically stable (positive-definite
    # Hessian of p, 0 <= cs2 <= 1): the table root is unique there
    Hm = np.zeros((n_rows, 4, 4))
    Hm[:, 0, 0] = fw[:, 16]
    for a_, c_ in ((1, 13), (2, 14), (3, 15)):
        Hm[:, 0, a_] = Hm[:, a_, 0] = fw[:, c_]
    Hm[:, 1, 1], Hm[:, 2, 2], Hm[:, 3, 3] = fw[:, 7], fw[:, 8], fw[:, 9]
    stable = (np.linalg.eigvalsh(Hm)[:, 0] > 0) & (fw[:, 6] >= 0) & (fw[:, 6] <= 1)
    del Hm
    err_T = np.abs(x[tab, 0] / x_true[tab, 0] - 1.0)
    err_mu = np.abs(x[tab, 1:] - x_true[tab, 1:]) * hb
    ts = tab & stable
    err_Ts = np.abs(x[ts, 0] / x_true[ts, 0] - 1.0)
    err_mus = np.abs(x[ts, 1:] - x_true[ts, 1:]) * hb
    # residual of the table rows against their targets
    fr = g.eos_thermo(0, x[tab])
    res = np.max(np.abs(np.column_stack([fr[:, 5], fr[:, 2], fr[:, 3], fr[:, 4]]) - tgt[tab]), axis=1)
    tl = stl == 0
    errl = np.abs(xl[tl & stable, 0] / x_true[tl & stable, 0] - 1.0)
    learned = {"value": n_rows / (msl * 1e-3), "unit": "inversions/s", "ms_per_batch": msl,
               "iterations": {"mean": float(itl.mean()), "p99": float(np.percentile(itl, 99)), "max": int(itl.max())},
               "table_rate": float(tl.mean()), "fallback_rate": float(np.mean(stl > 0)),
               "fail_rate": float(np.mean(stl < 0)),
               "recovered_rate": float(np.mean(tl & (np.abs(xl[:, 0] / x_true[:, 0] - 1.0) < 1e-8))),
               "p99_T_rel_err_stable_table_rows": float(np.percentile(errl, 99)),
               "training": {"samples": 5_000_000, "epochs": 20, "batch": 32768, "mse_standardised": mse,
                            "seconds": train_s},
               "what": "4-64-64-64-4 tanh MLP seed (BF16 tcgen05 kernels) for the table model, "
                       "then the reference seed chain"}
    # pre-inverted (s, rho) -> thermodynamics tables in the reference
    # generator's layout (decades 1e-3..1e2 in s, 1e-3..1e1 in rho, 20^4 nodes
    # a tile, 51.2M nodes). Generated here from the conformal-diagonal EoS,
    # which has a solution at every node (the generator aborts at a node
    # without one, and most nodes lie outside the synthetic table's domain).
    # Lookup throughput on the 2M states' (s, rho) against the entropy-mode
    # inversion of the same EoS from the generator's seed; accuracy on the rows
    # inside the tables.
    gc = api.GpuHydro(ics.RunConfig(eos_kind=1, thermo_mode=1))
    t0 = time.perf_counter()
    gc.preinverted_build()
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    sBSQ = np.ascontiguousarray(fw[:, [1, 2, 3, 4]])
    a_ = np.abs(sBSQ)
    cover = (a_[:, 0] >= 1e-3) & (a_[:, 0] < 1e2) & np.all((a_[:, 1:] >= 1e-3) & (a_[:, 1:] < 1e1), axis=1)
    q = torch.from_numpy(sBSQ).to(dev)
    look = torch.empty((n_rows, 11), dtype=torch.float64, device=dev)
    seedS = torch.tensor([750.0 / 197.0, 0, 0, 0], dtype=torch.float64, device=dev).repeat(n_rows, 1)
    xs = seedS.clone()
    ths = torch.empty((n_rows, 16), dtype=torch.float64, device=dev)
    sts = torch.empty(n_rows, dtype=torch.int32, device=dev)

    def timed_fn(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms_look = timed_fn(lambda: gc.preinverted_lookup_device(n_rows, q.data_ptr(), look.data_ptr(), stream.cuda_stream))

    def newton_s():
        xs.copy_(seedS)
        gc.eos_invert_device(1, 0, n_rows, q.data_ptr(), xs.data_ptr(), ths.data_ptr(), sts.data_ptr(), 0,
                             stream.cuda_stream)

    ms_newt = timed_fn(newton_s)
    lk, xn, okn = look.cpu().numpy(), xs.cpu().numpy(), sts.cpu().numpy() >= 0
    sel = cover & okn
    errT = np.abs(lk[sel, 0] / xn[sel, 0] - 1.0)
    preinv = {"value": n_rows / (ms_look * 1e-3), "unit": "lookups/s", "rows": n_rows, "ms_per_batch": ms_look,
              "newton_entropy_mode_same_eos": {"value": n_rows / (ms_newt * 1e-3), "unit": "inversions/s",
                                               "ms_per_batch": ms_newt, "solved_rate": float(okn.mean())},
              "generation": {"nodes": 5 * 4 * 4 * 4 * 20 ** 4, "seconds": gen_s, "eos": "conformal-diagonal",
                             "layout": "decades s 1e-3..1e2, rho 1e-3..1e1, 20^4 nodes a tile"},
              "rows_inside_tables": int(cover.sum()),
              "T_rel_err_inside": {"p50": float(np.median(errT)), "p99": float(np.percentile(errT, 99)),
                                   "max": float(errT.max())},
              "what": "multilinear lookup (reference EoS_Interpolator) vs Newton from T = 750/197 fm^-1, mu = 0"}
    gc.close()
    line = {"metric": "EoS inversions/s (2M states, synthetic 4-D table 151x41^3, energy mode)",
            "workload": "eos-table", "value": n_rows / (ms * 1e-3), "unit": "inversions/s",
            "ms_per_batch": ms, "rows": n_rows, "steps": args.steps, "warmup": args.warmup, "dtype": "f64",
            "seed": "reference chain (580 MeV forced seed, conformal-diagonal analytic seed)",
            "learned_seed": learned, "preinverted_tables": preinv,
            "iterations": {"mean": float(it.mean()), "p99": float(np.percentile(it, 99)), "max": int(it.max())},
            "table_rate": float(tab.mean()), "fallback_rate": float(np.mean(st > 0)),
            "fail_rate": float(np.mean(st < 0)),
            "stable_rate": float(stable.mean()),
            "max_err_table_rows": {"T_rel": float(err_T.max()), "mu_GeV": float(err_mu.max()),
                                   "p99_T_rel": float(np.percentile(err_T, 99)),
                                   "residual_fm": float(res.max())},
            "max_err_stable_table_rows": {"T_rel": float(err_Ts.max()), "mu_GeV": float(err_mus.max()),
                                          "p99_T_rel": float(np.percentile(err_Ts, 99))},
            "note": "rows in the band where this EoS is thermodynamically unstable (T ~ 0.10-0.19 GeV) "
                    "fail the reference's cs2 guard and fall back down the chain"}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py as O
        O.build()
        ot = O.OracleTable(n, lo, d, fields, conf5, cdiag5)
        m = min(n_rows, args.eos_cpu_rows)
        t0 = time.perf_counter()
        O.eos_invert_batch(rc, 0, tgt[:m], seeds=np.tile([580 / 197.3269804, 0, 0, 0], (m, 1)), table=ot)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": m / dt, "unit": "inversions/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"the first {m} rows, oracle/ OpenMP on {os.cpu_count()} threads"}
    print(json.dumps(line))


def run_hotspots3d(args):
    """3+1-D Milne viscous BSQ event: 120 x 120 x 100 (x, y, eta_s) lattice
    (1.44M particles), dx = 0.1 fm, deta = 0.06, h = 0.2 fm, 30 hot spots,
    shear eta/s = 0.08, bulk zeta/s peaked at T = 0.16 GeV, the synthetic
    tabulated EoS; RK2 steps in the mixed form (FP32 sums, FP64 state and
    EoS) and in the FP64 form, and the mixed form's error against the FP64
    form after the same steps."""
    import dataclasses
    import torch
    from ccake_gb300 import api, build, eos_table, ics
    build.build()
    p, rc = ics.hotspots_3d(n_xy=args.h3d_nxy, n_eta=args.h3d_neta, eos_kind=2, zeta_over_s=0.1)
    n, lo, d, fields = eos_table.synthetic_table()
    conf5, cdiag5 = api.table_fallback_scales(n, lo, d, fields, rc.freeze_out_T)
    steps = args.steps
    out = {}
    forms = (("mixed", 1), ("fp64", 0)) if args.form is None else ((args.form, 1 if args.form == "mixed" else 0),)
    for form, prec in forms:
        g = api.GpuHydro(dataclasses.replace(rc, precision=prec))
        g.set_eos_table(n, lo, d, fields, conf5, cdiag5)
        g.load(p)
        g.initialize()
        for _ in range(args.warmup):
            g.step(1)
        torch.cuda.synchronize()
        ms = g.step_timed(steps)
        out[form] = {"ms": ms, "state": {f: g.get(f) for f in ("e", "rhoB", "rhoQ", "T", "u0", "u2")},
                     "bytes": g.device_bytes(), "phase_ms": [float(v) for v in g.profile_phases(2)],
                     "eos_iters_mean": float(np.mean(g.get_int("eos_iters")))}
        g.close()
    if len(out) < 2:
        f0 = next(iter(out))
        print(json.dumps({"partial": True, "workload": "hotspots3d", "form": f0, "particles": p.n,
                          "ms_per_step": out[f0]["ms"] / steps, "phase_ms": out[f0]["phase_ms"],
                          "eos_iters_mean": out[f0]["eos_iters_mean"]}))
        return
    err = {}
    for f in ("e", "rhoB", "rhoQ", "T"):
        a, b = out["mixed"]["state"][f], out["fp64"]["state"][f]
        err[f] = float(np.max(np.abs(a - b) / (np.abs(b) + 1e-300)))
    for f in ("u0", "u2"):
        a, b = out["mixed"]["state"][f], out["fp64"]["state"][f]
        err[f + "_of_range"] = float(np.max(np.abs(a - b)) / (np.max(np.abs(b)) + 1e-300))
    npart = p.n
    line = {"metric": "particle-steps/s (3+1-D Milne viscous BSQ, tabulated EoS)", "workload": "hotspots3d",
            "value": npart * steps / (out["mixed"]["ms"] * 1e-3), "unit": "particle-steps/s",
            "form": "mixed (FP32 Kahan sums and EoM, FP64 EoS Newton, state and RK2)",
            "ms_per_step": out["mixed"]["ms"] / steps, "steps": steps, "warmup": args.warmup, "particles": npart,
            "fp64": {"value": npart * steps / (out["fp64"]["ms"] * 1e-3), "ms_per_step": out["fp64"]["ms"] / steps,
                     "phase_ms": out["fp64"]["phase_ms"], "eos_iters_mean": out["fp64"]["eos_iters_mean"]},
            "mixed_phase_ms": out["mixed"]["phase_ms"], "mixed_eos_iters_mean": out["mixed"]["eos_iters_mean"],
            "max_rel_err_mixed_vs_fp64": err, "device_bytes": out["mixed"]["bytes"],
            "config": {"lattice": f"{args.h3d_nxy}x{args.h3d_nxy}x{args.h3d_neta}", "dx_fm": 0.1, "deta": 0.06, "h_fm": 0.2, "eta_over_s": 0.08,
                       "zeta_over_s_peak": 0.1, "zeta_peak_T_GeV": 0.16, "eos": "synthetic table 151x41^3",
                       "dt": rc.dt, "tau0": rc.t0}}
    print(json.dumps(line))


def serve_events(n_events, seed=3, steps=100):
    """Events as the serving stream specifies (hot-spot count ~ U{10..60},
    particle count log-uniform in [10k, 400k] on a dx = 0.05 fm lattice,
    otherwise the 160k event's physics), each run for `steps` RK2 steps or
    until every particle is below the freeze-out temperature."""
    import dataclasses
    from ccake_gb300 import ics
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for j in range(n_events):
        npart = float(np.exp(rng.uniform(np.log(1e4), np.log(4e5))))
        side = max(20, int(round(np.sqrt(npart))))
        n_hot = int(rng.integers(10, 61))
        p, rc = ics.hotspots_2d(n_side=side, n_hot=n_hot, seed=int(rng.integers(1 << 31)))
        rc = dataclasses.replace(rc, particlization=1)   # stop when every particle froze out at 150 MeV
        out.append((p, rc, rc.t0 + steps * rc.dt))
    return out


def run_serve_replicated(args, world, rank):
    """The serving stream over N GPUs: every rank builds the same events, runs
    its share (by device bytes, ccake_gb300.replicas) on its own event
    server with the queue saturated, and rank 0 reports the aggregate
    events/h over the slowest rank's makespan."""
    import dataclasses
    import torch
    import torch.distributed as dist
    from ccake_gb300 import api, build, replicas
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    build.build()
    dist.init_process_group("nccl")
    evs = serve_events(args.serve_events, steps=args.steps)
    mixed = [(p, dataclasses.replace(rc, precision=1), tm) for p, rc, tm in evs]
    sizes = [p.n for p, _, _ in evs]

    def run_share(share):
        srv = api.Server(steps_per_launch=args.serve_quantum)
        if share:   # warm-up
            t = srv.submit(*share[0][1])
            srv.wait_all()
            srv.release(t)
        dist.barrier()
        t0 = time.perf_counter()
        tick = [(i, srv.submit(*ev)) for i, ev in share]
        srv.wait_all()
        span = time.perf_counter() - t0
        out = []
        for i, t in tick:
            r = srv.poll(t)
            r["makespan"] = span
            out.append((i, r))
            srv.release(t)
        srv.close()
        return out

    if not mixed:
        return
    # ranks with no event still join the barrier and the gather
    res = replicas.run_replicated(mixed, sizes, rank, world, run_share, dist)
    dist.destroy_process_group()
    if rank != 0:
        return
    span = max(r["makespan"] for r in res)
    psteps = sum(r["particles"] * r["steps"] for r in res)
    print(json.dumps({"metric": "events/h (serving stream, continuous batching, mixed form)", "workload": "serve",
                      "value": 3600.0 * len(res) / span, "unit": "events/h", "n_gpus": world,
                      "events": len(res), "steps_per_event": args.steps, "scaling": "strong",
                      "failed": sum(r["state"] != "done" for r in res),
                      "particle_steps_per_s": psteps / span, "makespan_s": span,
                      "parallelism": f"replicas{world}: events split by device bytes, one event server per GPU"}))


def run_serve(args):
    """Serving stream on one GPU through ccake_server_*: capacity with the
    queue saturated, then Poisson arrivals at 80 % of that capacity (p50/p99
    latency, events/h), and a subset of the same events run one at a time in
    the plain FP64 form."""
    import dataclasses
    from ccake_gb300 import api, build
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        run_serve_replicated(args, world, int(os.environ.get("RANK", "0")))
        return
    build.build()
    n_ev = args.serve_events
    evs = serve_events(n_ev, steps=args.steps)
    mixed = [(p, dataclasses.replace(rc, precision=1), tm) for p, rc, tm in evs]
    psteps = sum(p.n * args.steps for p, _, _ in evs)
    # warm-up: one small event through a server (build, first graph capture)
    srv = api.Server(steps_per_launch=args.serve_quantum)
    t = srv.submit(mixed[0][0], mixed[0][1], mixed[0][2])
    srv.wait_all()
    srv.release(t)
    # 1. capacity: every event submitted at once
    t0 = time.perf_counter()
    tickets = [srv.submit(p, rc, tm) for p, rc, tm in mixed]
    srv.wait_all()
    makespan = time.perf_counter() - t0
    res = [srv.poll(t) for t in tickets]
    for t in tickets:
        srv.release(t)
    failed = sum(r["state"] != "done" for r in res)
    frozen = sum(r["frozen"] for r in res)
    psteps = sum(r["particles"] * r["steps"] for r in res)
    capacity = n_ev / makespan
    # 2. Poisson arrivals at 80 % of capacity
    rng = np.random.Generator(np.random.PCG64(3))
    gaps = rng.exponential(1.0 / (0.8 * capacity), n_ev)
    t_start = time.perf_counter()
    tickets = []
    next_t = t_start
    for (p, rc, tm), gap in zip(mixed, gaps):
        next_t += gap
        while time.perf_counter() < next_t:
            time.sleep(min(1e-3, max(0.0, next_t - time.perf_counter())))
        tickets.append(srv.submit(p, rc, tm))
    srv.wait_all()
    wall = time.perf_counter() - t_start
    res2 = [srv.poll(t) for t in tickets]
    for t in tickets:
        srv.release(t)
    srv.close()
    lat = np.array([r["latency_s"] for r in res2])
    que = np.array([r["queue_s"] for r in res2])
    # 3. the same events one at a time, plain FP64 form, on a subset
    sub = evs[:args.serve_fp64_events]
    t0 = time.perf_counter()
    for p, rc, tm in sub:
        g = api.GpuHydro(rc)
        g.load(p)
        g.initialize()
        g.step(args.steps)
        g.close()
    fp64_each = (time.perf_counter() - t0) / len(sub)
    line = {"metric": "events/h (serving stream, continuous batching, mixed form)", "workload": "serve",
            "value": 3600.0 * n_ev / makespan, "unit": "events/h",
            "events": n_ev, "steps_per_event": args.steps, "failed": failed, "stopped_by_freeze_out": frozen,
            "particle_steps_per_s": psteps / makespan, "makespan_s": makespan,
            "poisson": {"rate_events_per_s": 0.8 * capacity, "wall_s": wall,
                        "events_per_h": 3600.0 * n_ev / wall,
                        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                      "max": float(lat.max())},
                        "queue_s": {"p50": float(np.percentile(que, 50)), "p99": float(np.percentile(que, 99))},
                        "failed": sum(r["state"] != "done" for r in res2)},
            "one_at_a_time_fp64": {"events": len(sub), "seconds_per_event": fp64_each,
                                   "events_per_h": 3600.0 / fp64_each},
            "config": {"events": "hot spots ~ U{10..60}, particles log-uniform in [10k, 400k] (dx = 0.05 fm "
                                 "lattice), conformal-diagonal EoS, eta/s = 0.08, dt = 0.001 fm/c",
                       "stop": f"{args.steps} RK2 steps or every particle frozen out (freeze-out status "
                               f"machine at T = 150 MeV)",
                       "scaled": "runs are capped at the given steps (to freeze-out or 10 fm/c an event takes "
                                 "~9000 steps at this dt)",
                       "server": {"steps_per_launch": args.serve_quantum, "hbm_budget": "80% of free memory"}}}
    print(json.dumps(line))


def run_form_only(args, form):
    """Only the timed step loop of one precision form (for profiler launch
    lists); prints a partial line."""
    import dataclasses
    import torch
    from ccake_gb300 import api, build
    build.build()
    p, rc = workload()
    rc = dataclasses.replace(rc, precision=1 if form == "mixed" else 0)
    if args.diffusion:
        # the diffusion sector on the same event: B and Q diffuse with
        # kappa/T^2 = 0.3 (the event carries no strangeness)
        rc = dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=(0.3, 0, 0, 0, 0, 0, 0, 0, 0.3))
    g = api.GpuHydro(rc)
    g.load(p)
    g.initialize()
    for _ in range(args.warmup):
        g.step(1)
    torch.cuda.synchronize()
    ms = g.step_timed(args.steps)
    metric = METRIC if form == "fp64" else METRIC.replace("plain FP64", "mixed precision")
    line = {"partial": True, "form": form, "diffusion": bool(args.diffusion), "metric": metric, "unit": UNIT,
            "steps": args.steps, "ms_per_step": ms / args.steps, "value": p.n * args.steps / (ms * 1e-3)}
    if args.diffusion and not args.no_cpu:
        steps = max(1, args.ref_steps)
        value, dt, _ = cpu_reference(p, rc, steps, warmup=1)
        line["cpu_port"] = {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                            "sample": f"{steps} RK2 steps after 1 warm-up step, all {p.n} particles, "
                                      "diffusion on"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--ref-steps", type=int, default=4, help="RK2 steps timed on the CPU (--form --diffusion)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", choices=["hotspots", "eos-table", "hotspots3d", "serve"], default="hotspots",
                    help="hotspots: the 160k hot-spot event (default); eos-table: the EoS-inversion stress test; "
                         "hotspots3d: the 1.44M-particle 3+1-D event; serve: the serving stream")
    ap.add_argument("--h3d-nxy", type=int, default=120)
    ap.add_argument("--h3d-neta", type=int, default=100)
    ap.add_argument("--serve-events", type=int, default=64)
    ap.add_argument("--serve-quantum", type=int, default=20)
    ap.add_argument("--serve-fp64-events", type=int, default=8)
    ap.add_argument("--eos-rows", type=int, default=2_000_000)
    ap.add_argument("--eos-cpu-rows", type=int, default=20_000)
    ap.add_argument("--form", choices=["fp64", "mixed"], default=None,
                    help="time only this form's step loop (profiler launch lists); partial output")
    ap.add_argument("--diffusion", action="store_true",
                    help="with --form fp64: the diffusion sector on (kappa/T^2 = 0.3 for B and Q)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "eos-table":
        run_eos_table(args)
    elif args.workload == "hotspots3d":
        run_hotspots3d(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.form:
        run_form_only(args, args.form)
    else:
        run_ours(args, world, rank)


if __name__ == "__main__":
    main()
