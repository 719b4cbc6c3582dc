"""Algorithmic traffic and arithmetic of the SPH step (the roofline inputs).

Rule: compulsory HBM traffic of a two-pass fused design. Every per-particle
FP64 scalar one derivative evaluation must read or write is counted once at
8 B; neighbour reads count 0 (tile reuse); cell-sort keys 8 B per particle
per build. The field lists are the ones the passes of this library touch:

  pass A (smoothing + EoS):  read the state and the EoS seed, write the LRF
                             densities and the thermodynamics;
  pass B (gradients + EoM + RK2): read positions, velocities, pass-A outputs,
                             the state and the step-start cache, write the state.

`python -m ccake_gb300.traffic_model` writes traffic_model.json beside this
file (the committed copy), with the pair-slot counts of `pair_slots` on the
benchmark lattices.
"""
from __future__ import annotations

import json
import os

SCALAR = 8   # bytes per FP64 scalar

# per-substep field lists (names of FP64 scalars per particle)
FIELDS = {
    "C1": {   # 2-D ideal, no charges (Gubser)
        "binning": ["x", "y", "key"],
        "passA": ["x", "y", "u_x", "u_y", "ext_s", "T_seed",
                  "sigma_lab", "s_star", "T", "p", "w", "dwds", "cs2"],
        "passB": ["x", "y", "u_x", "u_y", "p", "sigma_lab", "w", "dwds", "s", "T", "ext_s",
                  "y0_x", "y0_y", "y0_ux", "y0_uy", "y0_s",
                  "y_x", "y_y", "y_ux", "y_uy", "y_s"],
        "step_extra": ["y0_x", "y0_y", "y0_ux", "y0_uy", "y0_s"],
    },
    "C2": {   # 2-D viscous, B/S/Q, shear (the bench event)
        "binning": ["x", "y", "key"],
        "passA": ["x", "y", "u_x", "u_y", "ext_s", "ext_B", "ext_S", "ext_Q", "T_seed", "muB_seed", "muQ_seed",
                  "muS_seed",
                  "sigma_lab", "s_star", "B_star", "S_star", "Q_star", "T", "muB", "muQ", "muS", "p", "e", "w",
                  "cs2", "dwds", "dwdB", "dwdS"],
        "passB": ["x", "y", "u_x", "u_y", "p", "e", "sigma_lab", "ext_Pi", "ext_pi11", "ext_pi12",
                  "T", "muB", "muQ", "muS", "rhoB", "rhoS", "rhoQ", "s", "w", "cs2", "dwds", "dwdB", "dwdS", "dwdQ",
                  "st_x", "st_y", "st_ux", "st_uy", "st_s", "st_B", "st_S", "st_Q", "st_Pi", "st_pi11", "st_pi12",
                  "st_pi22",
                  "y0_x", "y0_y", "y0_ux", "y0_uy", "y0_s", "y0_B", "y0_S", "y0_Q", "y0_Pi", "y0_pi11", "y0_pi12",
                  "y0_pi22",
                  "y_x", "y_y", "y_ux", "y_uy", "y_s", "y_B", "y_S", "y_Q", "y_Pi", "y_pi11", "y_pi12", "y_pi22"],
        "step_extra": ["y0_x", "y0_y", "y0_ux", "y0_uy", "y0_s", "y0_B", "y0_S", "y0_Q", "y0_Pi", "y0_pi11",
                       "y0_pi12", "y0_pi22"],
    },
}

# FP64 operations (an FMA counts 2) of the FP64 form per particle and launch.
# C2 (the bench event) from the kernels' FP64 instructions, counted in the
# source and checked against ncu (2 DFMA + DMUL + DADD per launch over the
# 160k particles: pass A smoothing 1511, EoS 481, pass B 3873):
#   pair_A  31 = displacement 2 + exact |d|^2 3 + kernel values + 5 sums 10;
#                the kernel values cost 23 with both branches (1/r by the
#                refined FP32 estimate, W and grad-W of q < 1 and q >= 1)
#                and 13 or 15 when the warp's lanes agree on one branch,
#                which the ordered candidate lists make the common case
#                (31 is the measured mean)
#   pair_B  43 = m fg 1 + displacement 2 + m grad W 2 + 9 separable sums with
#                shear (S1, SP, SE, SB, SV, S0, SD) 38
#   particle_A  gamma, v and the LRF densities; eos the inversion and the
#   records; eom the transport, MRF equations of motion and RK2 update.
# C1 and C4 are estimates of the same kind (no shear and charges in C1; 3-D,
# table EoS and bulk in C4).
FLOPS = {
    "C1": {"neighbours": 48, "pair_A": 38, "pair_B": 27, "particle_A": 60, "eos": 250, "eom": 700},
    "C2": {"neighbours": 46, "pair_A": 31, "pair_B": 43, "particle_A": 60, "eos": 490, "eom": 1910},
    "C4": {"neighbours": 447, "pair_A": 40, "pair_B": 60, "particle_A": 80, "eos": 1200, "eom": 2500},
}

# 3-D: +1 position, +1 velocity, +2 shear components per state copy
C4_BYTES_PER_PARTICLE_STEP = 1900


def scalars(config: str, part: str) -> int:
    return len(FIELDS[config][part])


def bytes_per_launch(config: str, kernel: str, n: int) -> int:
    """Algorithmic bytes of one launch of `kernel` ("binning", "passA",
    "passB") over n particles."""
    return scalars(config, kernel) * SCALAR * n


def bytes_per_particle_step(config: str) -> int:
    if config == "C4":
        return C4_BYTES_PER_PARTICLE_STEP
    f = FIELDS[config]
    per_sub = len(f["binning"]) + len(f["passA"]) + len(f["passB"])
    return (2 * per_sub + len(f["step_extra"])) * SCALAR


def flops_per_particle_step(config: str) -> int:
    c = FLOPS[config]
    return 2 * (c["neighbours"] * (c["pair_A"] + c["pair_B"]) + c["particle_A"] + c["eos"] + c["eom"])


def flops_per_launch(config: str, kernel: str, n: int) -> float:
    """FP64 operations of one pass launch over n particles: pass A (the
    smoothing kernel and the EoS kernel) and pass B (gradients, EoM, RK2)."""
    c = FLOPS[config]
    if kernel == "passA":
        return n * (c["neighbours"] * c["pair_A"] + c["particle_A"] + c["eos"])
    if kernel == "passB":
        return n * (c["neighbours"] * c["pair_B"] + c["eom"])
    return 0.0


def pair_slots(pts, h, skin_frac=0.1, warp=32, icl=8, jcl=4, sample=37):
    """Pair slots a lane walks per particle under four pair-loop designs, on
    the particle positions `pts` (n x D) with smoothing length h, for interior
    particles (at least the median count within 2h):

      in_2h        pairs within 2h (the useful work)
      candidates   the candidate list within 2h + skin (this library)
      stencil      the 3^D cells of edge >= 2h + skin around the particle's cell
      warp_union   the union of the stencils of a warp of 32 consecutive
                   cell-sorted particles (a warp-uniform loop over staged tiles)
      cluster      i-clusters of 8 x j-clusters of 4 consecutive cell-sorted
                   particles whose bounding boxes lie within 2h + skin, per
                   i-particle (a lane per (i, j) pair, sums reduced by shuffles)

    Counted with a k-d tree (scipy); warps and clusters are sampled."""
    import numpy as np
    from scipy.spatial import cKDTree
    n, D = pts.shape
    cut, cutc = 2 * h, 2 * h * (1 + skin_frac)
    tree = cKDTree(pts)
    nin = np.array([len(l) - 1 for l in tree.query_ball_point(pts, cut * (1 + 1e-12))])
    ncand = np.array([len(l) - 1 for l in tree.query_ball_point(pts, cutc)])
    lo = pts.min(0)
    span = pts.max(0) - lo
    ncell = np.maximum(np.floor(span / cutc).astype(int), 1)
    c = np.minimum(np.floor((pts - lo) / (span / ncell)).astype(int), ncell - 1)
    lin = np.ravel_multi_index(c.T[::-1], ncell[::-1])
    order = np.argsort(lin, kind="stable")
    counts = np.bincount(lin, minlength=int(np.prod(ncell))).reshape(ncell[::-1])
    pad = np.pad(counts, 1)
    st = np.zeros_like(counts)
    for off in np.ndindex(*([3] * D)):
        st += pad[tuple(slice(o, o + s) for o, s in zip(off, counts.shape))]
    stencil = st.ravel()[lin]
    cidx = np.array(np.unravel_index(lin[order], ncell[::-1])).T
    wu = []
    for w0 in range(0, n, warp * sample):
        nb = set()
        for x in {tuple(v) for v in cidx[w0:w0 + warp]}:
            for off in np.ndindex(*([3] * D)):
                y = tuple(a + o - 1 for a, o in zip(x, off))
                if all(0 <= a < s for a, s in zip(y, counts.shape)):
                    nb.add(y)
        wu.append(sum(int(counts[y]) for y in nb))
    ps = pts[order]

    def boxes(k):
        b = ps[:(n // k) * k].reshape(-1, k, D)
        return b.min(1), b.max(1)
    ilo, ihi = boxes(icl)
    jlo, jhi = boxes(jcl)
    jt = cKDTree((jlo + jhi) / 2)
    reach = cutc + (np.max(np.linalg.norm(ihi - ilo, axis=1)) + np.max(np.linalg.norm(jhi - jlo, axis=1))) / 2
    slots = []
    for a in range(0, len(ilo), sample):
        cand = jt.query_ball_point((ilo[a] + ihi[a]) / 2, reach)
        gap = np.maximum(0, np.maximum(jlo[cand] - ihi[a], ilo[a] - jhi[cand]))
        slots.append(int(np.sum(np.sum(gap * gap, 1) <= cutc * cutc)) * jcl)
    inner = nin >= np.percentile(nin, 50)
    return {"in_2h": float(nin[inner].mean()), "candidates": float(ncand[inner].mean()),
            "stencil": float(stencil[inner].mean()), "warp_union": float(np.mean(wu)),
            "cluster": float(np.mean(slots)), "particles_per_cell": float(n / np.prod(ncell))}


def bench_lattices():
    """The 2-D hot-spot lattice (400 x 400, dx 0.05 fm, h 0.1 fm) and the 3-D
    Milne lattice (120 x 120 x 100, dx 0.1 fm, d eta 0.06, h 0.2)."""
    import numpy as np
    xs = -10 + 0.05 * np.arange(400)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    xs3 = -6 + 0.1 * np.arange(120)
    es = -3 + 0.06 * np.arange(100)
    E, Y3, X3 = np.meshgrid(es, xs3, xs3, indexing="ij")
    return {"C2": (np.column_stack([X.ravel(), Y.ravel()]), 0.1),
            "C4": (np.column_stack([X3.ravel(), Y3.ravel(), E.ravel()]), 0.2)}


def as_dict(with_slots=False):
    d = {"rule": "compulsory FP64 scalars x 8 B per particle per launch; neighbour reads 0; keys 8 B",
         "fields": FIELDS, "flops": FLOPS,
         "bytes_per_particle_step": {c: bytes_per_particle_step(c) for c in ("C1", "C2", "C4")},
         "flops_per_particle_step": {c: flops_per_particle_step(c) for c in ("C1", "C2", "C4")}}
    if with_slots:
        d["pair_slots"] = {k: {a: round(b, 1) for a, b in pair_slots(*v).items()}
                           for k, v in bench_lattices().items()}
    return d


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "traffic_model.json")
    with open(path, "w") as fh:
        json.dump(as_dict(with_slots=True), fh, indent=1)
        fh.write("\n")
    print(path)
