// Kernels of the GB300 SPH hot path.
//
// One RK2 substep is two passes over each particle's neighbours:
//   pass A  (per particle a): smoothing sums over the candidate list, the
//           exact 2h neighbour list with its grad-W factors, LRF densities;
//           then (thermo.cu) the EoS Newton inversion, pi^{mu nu}
//           constraints and neighbour record B.
//   pass B  (per particle a): gradient sums in separable form, the MRF
//           equations of motion and the RK2 update of the state; writes
//           neighbour record A for the next substep.
// Each particle's sums are accumulated in registers by the thread that owns
// it (gather, no atomics), in a fixed cell/index order, so results are
// reproducible run to run.
#include <climits>
#include <cstdio>

#include "kernels.cuh"
#include "passes.cuh"
#include "physics.cuh"

namespace ccake {

namespace {

using namespace passes;

// ---------------------------------------------------------------------------
// neighbour cells: count, scan, scatter, in-cell sort
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_bin(RunConst rc, Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const Grid& g = rc.grid;
  int c = cell_coord(g, 0, p.y[Y_X0 * p.n + i]);
  c += g.nc[0] * cell_coord(g, 1, p.y[Y_X1 * p.n + i]);
  if (D == 3) c += g.nc[0] * g.nc[1] * cell_coord(g, 2, p.y[Y_X2 * p.n + i]);
  p.cell_of[i] = c;
  p.cell_rank[i] = atomicAdd(&p.cell_count[c], 1);
}

// Exclusive scan of the cell counts, multi-CTA: each CTA scans a tile of
// kScanTile cells (coalesced through shared memory) into cell_start and
// publishes the tile total; the last CTA to finish (atomic ticket, no
// waiting) scans the tile totals into tile offsets; k_scan_add adds them.
constexpr int kScanThreads = 256;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanThreads * kScanPer;

__device__ __forceinline__ int32_t block_exclusive_scan(int32_t x, int32_t* warp_tot, int32_t* total) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  int32_t v = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) warp_tot[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int32_t w = (lane < nw) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) warp_tot[lane] = w;
  }
  __syncthreads();
  const int32_t excl = v - x + (wid > 0 ? warp_tot[wid - 1] : 0);
  if (total) *total = warp_tot[nw - 1];
  __syncthreads();
  return excl;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int32_t* __restrict__ cnt, int32_t* __restrict__ start,
                                                             int32_t* __restrict__ aux, int ncell) {
  __shared__ int32_t sh[kScanTile];
  __shared__ int32_t warp_tot[32];
  __shared__ int32_t tile_total;
  __shared__ bool last;
  const int tid = threadIdx.x;
  const int base = blockIdx.x * kScanTile;
#pragma unroll
  for (int j = 0; j < kScanPer; j++) {
    const int c = base + j * kScanThreads + tid;
    sh[j * kScanThreads + tid] = c < ncell ? cnt[c] : 0;
  }
  __syncthreads();
  int32_t v[kScanPer], sum = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; j++) {
    v[j] = sh[tid * kScanPer + j];
    sum += v[j];
  }
  int32_t run = block_exclusive_scan(sum, warp_tot, &tile_total);
#pragma unroll
  for (int j = 0; j < kScanPer; j++) {
    sh[tid * kScanPer + j] = run;
    run += v[j];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kScanPer; j++) {
    const int c = base + j * kScanThreads + tid;
    if (c < ncell) start[c] = sh[j * kScanThreads + tid];
  }
  // aux: [0, ntiles) tile totals, then tile offsets, then the ticket
  const int ntiles = gridDim.x;
  int32_t* tot = aux;
  int32_t* off = aux + ntiles;
  int32_t* ticket = aux + 2 * ntiles;
  if (tid == 0) {
    tot[blockIdx.x] = tile_total;
    __threadfence();
    last = (atomicAdd(ticket, 1) == ntiles - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  int32_t carry = 0;
  for (int t0 = 0; t0 < ntiles; t0 += kScanThreads) {
    const int t = t0 + tid;
    const int32_t x = t < ntiles ? ((volatile int32_t*)tot)[t] : 0;
    int32_t chunk;
    const int32_t e = block_exclusive_scan(x, warp_tot, &chunk);
    if (t < ntiles) off[t] = carry + e;
    carry += chunk;
  }
  if (tid == 0) {
    start[ncell] = carry;
    *ticket = 0;
  }
}

__global__ void k_scan_add(int32_t* __restrict__ start, const int32_t* __restrict__ aux, int ncell, int ntiles) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int tile = c / kScanTile;
  if (tile > 0) start[c] += aux[ntiles + tile];
}

__global__ void k_scatter(Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  p.cell_idx[p.cell_start[p.cell_of[i]] + p.cell_rank[i]] = i;
}

// Sorts each cell's index list (one warp a cell; rank of a value = number of
// smaller values, by shuffles) so that the summation order does not depend on
// the atomic arrival order. Cells of more than 32 kSortChunks particles fall
// back to one lane's insertion sort.
constexpr int kSortChunks = 8;
__global__ void k_sort_cells(Ptrs p, int ncell) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncell) return;
  const int b = p.cell_start[warp], e = p.cell_start[warp + 1];
  const int m = e - b;
  if (m <= 1) return;
  if (m > 32 * kSortChunks) {
    if (lane == 0)
      for (int j = b + 1; j < e; j++) {
        const int32_t key = p.cell_idx[j];
        int k = j - 1;
        while (k >= b && p.cell_idx[k] > key) { p.cell_idx[k + 1] = p.cell_idx[k]; k--; }
        p.cell_idx[k + 1] = key;
      }
    return;
  }
  const int nch = (m + 31) >> 5;
  int32_t v[kSortChunks];
  int r[kSortChunks];
#pragma unroll
  for (int c = 0; c < kSortChunks; c++) {
    const int j = c * 32 + lane;
    v[c] = (c < nch && j < m) ? p.cell_idx[b + j] : INT_MAX;
    r[c] = 0;
  }
#pragma unroll
  for (int c2 = 0; c2 < kSortChunks; c2++) {
    if (c2 >= nch) break;
    for (int k = 0; k < 32; k++) {
      const int32_t u = __shfl_sync(0xffffffffu, v[c2], k);
#pragma unroll
      for (int c = 0; c < kSortChunks; c++) r[c] += (u < v[c]) ? 1 : 0;
    }
  }
  __syncwarp();
#pragma unroll
  for (int c = 0; c < kSortChunks; c++) {
    const int j = c * 32 + lane;
    if (c < nch && j < m) p.cell_idx[b + r[c]] = v[c];
  }
}

// Candidate (Verlet) list of particle i: every b != i in the 3^D cells around
// it whose FP32 squared distance is not above (2h + skin)^2 by more than its
// error bound (so no pair within 2h + skin in FP64 is dropped). In the FP64
// form the list is in three parts by the FP32 distance at the build, each in
// cell order: the pairs with r < 0.9 h, those with 0.9 h <= r < 1.1 h, then
// the rest. The lanes of a warp then mostly reach pairs on the same side of
// r = h together in the FP64 pair loop (on a lattice with h = 2 dx, r = h
// exactly is a lattice distance: those pairs, on either side as the
// particles move, are kept together in the middle part). The mixed form's
// FP32 loops gain nothing from it and gather better in plain cell order,
// which they keep. With Kc = 0 it only counts. The
// largest count goes to cand_max (zeroed before the build): the host grows
// the capacities when it exceeds them and builds again, so no entry past Kc is
// ever used.
template <int D>
__global__ void __launch_bounds__(kBlock) k_candidates(RunConst rc, Ptrs p) {
  const int i_ = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i_ < p.n;
  const int i = live ? i_ : 0;
  const int n = p.n;
  const double xa[3] = {p.y[Y_X0 * n + i], p.y[Y_X1 * n + i], D == 3 ? p.y[Y_X2 * n + i] : 0.0};
  const float4 pa = p.posf[i];
  const float cut2f = rc.fcutc2 * 1.000001f;
  const float h2lo = 0.2025f * rc.fcut2, h2hi = 0.3025f * rc.fcut2;   // (0.9 h)^2, (1.1 h)^2
  int rlo[D == 3 ? 9 : 3], rhi[D == 3 ? 9 : 3];
  const int nr = live ? neighbour_ranges<D>(rc.grid, p.cell_start, xa, rlo, rhi) : 0;
  const int Kc = p.Kc;
  int c = 0;
  const int nparts = rc.cfg.precision == 0 ? 3 : 1;
#pragma unroll 1
  for (int part = 0; part < nparts; part++)
    for (int r = 0; r < nr; r++)
      for (int j = rlo[r]; j < rhi[r]; j++) {
        const int b = p.cell_idx[j];
        if (b == i) continue;
        float d2f, bound;
        if (!maybe_neighbour<D>(pa, __ldg(&p.posf[b]), cut2f, d2f, bound)) continue;
        if (nparts > 1 && (d2f < h2lo ? 0 : (d2f < h2hi ? 1 : 2)) != part) continue;
        if (c < Kc) p.cand_idx[(size_t)c * n + i] = b;
        c++;
      }
  // every lane reaches the warp reduction; lanes past the end count 0
  if (!live) c = 0;
  const int wmax = __reduce_max_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && p.cand_max) atomicMax(p.cand_max, wmax);
  if (live) p.cand_cnt[i] = c;
}

// Iterates the 3^D neighbour cells of a position; calls f(b) for every
// particle b != a in them.
template <int D, class F>
__device__ __forceinline__ void for_candidates(const RunConst& rc, const Ptrs& p, int a, const double* xa, F&& f) {
  const Grid& g = rc.grid;
  const int cx = cell_coord(g, 0, xa[0]), cy = cell_coord(g, 1, xa[1]);
  const int cz = (D == 3) ? cell_coord(g, 2, xa[2]) : 0;
  const int zlo = (D == 3) ? max(cz - 1, 0) : 0, zhi = (D == 3) ? min(cz + 1, g.nc[2] - 1) : 0;
  for (int z = zlo; z <= zhi; z++)
    for (int y = max(cy - 1, 0); y <= min(cy + 1, g.nc[1] - 1); y++) {
      const int row = (z * g.nc[1] + y) * g.nc[0];
      const int c0 = row + max(cx - 1, 0), c1 = row + min(cx + 1, g.nc[0] - 1);
      // cells c0..c1 are contiguous in the sorted list
      const int jb = p.cell_start[c0], je = p.cell_start[c1 + 1];
      for (int j = jb; j < je; j++) {
        const int b = p.cell_idx[j];
        if (b != a) f(b);
      }
    }
}

// ---------------------------------------------------------------------------
// pass A
// ---------------------------------------------------------------------------
// The smoothing kernel carries no EoS code: the inversion's ~255 registers
// would cap it at 8 warps an SM, and its pair loop, bound by the FP64 pipe,
// runs better with more warps to draw FP64 instructions from; k_thermo runs
// the inversion right after it.
template <int D>
__global__ void __launch_bounds__(kBlock) k_passA(RunConst rc, Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double t = p.clock->t;
  const double2* ra = reinterpret_cast<const double2*>(p.recA);
  const double2 a01 = ra[(size_t)i * 4 + 0], a23 = ra[(size_t)i * 4 + 1];
  const double2 a45 = ra[(size_t)i * 4 + 2], a67 = ra[(size_t)i * 4 + 3];
  const double xa[3] = {a01.x, a01.y, a23.x};
  const double k0 = rc.k0;
  double sl = a23.y * k0, s0 = a45.x * k0, s1 = a45.y * k0, s2 = a67.x * k0, s3 = a67.y * k0;
  int nn = 0;
  const int K = p.K;
  // Two phases per chunk of candidates, so that the FP64 work runs with full
  // warps (an FP64 warp instruction costs the same pipe time whatever its
  // active-lane count): phase 1 screens candidates in FP32 and keeps the
  // survivors in this thread's shared-memory column; phase 2 runs the exact
  // FP64 predicate, W and the grad-W factor on the survivors.
  __shared__ int32_t surv[kSurv][kBlock];
  const int tid = threadIdx.x;
  const float4 pa = p.posf[i];
  const float cut2f = rc.fcut2 * 1.000001f;
  // the candidate list of the last build holds every b that can be within
  // 2h now
  const int nc = min(p.cand_cnt[i], p.Kc);
  // the factorised 3-D kernel (the reference's factorized_kernel option)
  const bool fact = (D == 3) && rc.cfg.factorized_kernel;
  int kk = 0;
  while (kk < nc) {
    int ns = 0;
    while (kk < nc && ns < kSurv) {           // phase 1 (FP32)
      const int b = p.cand_idx[(size_t)kk * n + i];
      kk++;
      const float4 pb = __ldg(&p.posf[b]);
      // the screen never drops a pair the exact predicate below accepts, so
      // the neighbour set is the FP64 one
      float d2f, bound;
      if (!maybe_neighbour<D>(pa, pb, cut2f, d2f, bound)) continue;
      surv[ns++][tid] = b;
    }
    for (int s = 0; s < ns; s++) {            // phase 2 (FP64)
      const int b = surv[s][tid];
      const double2 b01 = __ldg(&ra[(size_t)b * 4 + 0]), b23 = __ldg(&ra[(size_t)b * 4 + 1]);
      double d[3] = {xa[0] - b01.x, xa[1] - b01.y, (D == 3) ? xa[2] - b23.x : 0.0};
      const double d2 = dist2_exact<D>(d);
      // d2 <= (2h)^2 on the integer pipe: d2 is a sum of squares (+0 or
      // more), whose IEEE bits read as an unsigned integer order like the
      // value, and a NaN of either sign compares above the cut
      if ((unsigned long long)__double_as_longlong(d2) > rc.cut2_bits) continue;
      double W, fg, fe = 0.0;
      if (fact) {
        // W_2D(r_perp, hT) W_1D(|d eta|, hEta) and its gradient
        // (src/kernel.cpp:129-170): (dW_2D W_1D along d_perp, W_2D dW_1D
        // along d eta)
        double W2, g2, W1, g1;
        pair_kernel(rc.kperp, d[0] * d[0] + d[1] * d[1], W2, g2);
        pair_kernel(rc.keta, d[2] * d[2], W1, g1);
        W = W2 * W1;
        fg = g2 * W1;
        fe = W2 * g1;
      } else {
        pair_kernel_warp(rc, d2, W, fg);
      }
      if (nn < K) {
        p.nbr_idx[(size_t)nn * n + i] = b;
        p.nbr_f[(size_t)nn * n + i] = fg;
        if (fact) p.nbr_fe[(size_t)nn * n + i] = fe;
      }
      nn++;
      const double2 b45 = __ldg(&ra[(size_t)b * 4 + 2]);
      const double2 b67 = __ldg(&ra[(size_t)b * 4 + 3]);
      sl += b23.y * W;
      s0 += b45.x * W;
      s1 += b45.y * W;
      s2 += b67.x * W;
      s3 += b67.y * W;
    }
  }
  if (nn > K) flag_error(p.err, E_NBR_OVERFLOW);
  // gamma and v from u (update_velocity), LRF densities (get_LRF: lab/(gamma t)
  // in Milne coordinates, lab/gamma in Cartesian ones)
  const double tm = rc.cfg.coord == 1 ? 1.0 : t;
  const double u3[3] = {p.y[Y_U0 * n + i], p.y[Y_U1 * n + i], D == 3 ? p.y[Y_U2 * n + i] : 0.0};
  const double g = gamma_milne<D>(u3, tm * tm);
  p.gam[i] = g;
  // two divisions instead of twelve (an FP64 division is a long sequence on
  // the FP64 pipe): 1/gamma and 1/(gamma tau)
  const double ig = 1.0 / g, igt = 1.0 / (g * tm);
#pragma unroll
  for (int q = 0; q < 3; q++) p.v[q * n + i] = (q < D) ? u3[q] * ig : 0.0;
  p.slab[i] = sl;
  p.sig[i] = sl * igt;
  p.th[T_S * n + i] = s0 * igt;
  p.th[T_RB * n + i] = s1 * igt;
  p.th[T_RS * n + i] = s2 * igt;
  p.th[T_RQ * n + i] = s3 * igt;
  p.btrack[i] = nn;
}

// Diffusion sums of src/sph_workstation.cpp:909-967 over the list pass A
// wrote, for particle a: v.grad q^0_c = sl_a sum_b m_b (v_a . grad W)
// (q^0_b / sl_b^2 + q^0_a / sl_a^2), div q_c = sl_a sum_b m_b grad_k W
// (q^k_b / sl_b^2 + q^k_a / sl_a^2) and grad_k alpha_c = sum_b (m_b / sl_a)
// (alpha_b - alpha_a) grad_k W, in the separable form of pass B.
template <int D>
__global__ void __launch_bounds__(kBlock) k_diffgrad(Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double* rbA = p.recB + (size_t)i * RB;
  const double xa[3] = {rbA[B_X0], rbA[B_X1], rbA[B_X2]};
  double S1[D], SQ0[3][D], SA[3][D], SQI[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < D; k++) {
    S1[k] = 0.0;
#pragma unroll
    for (int c = 0; c < 3; c++) SQ0[c][k] = SA[c][k] = 0.0;
  }
  const int cnt = min(p.btrack[i], p.K);
  for (int kk = 0; kk < cnt; kk++) {
    const int b = p.nbr_idx[(size_t)kk * n + i];
    const double fg = p.nbr_f[(size_t)kk * n + i];
    const double* rb = p.recB + (size_t)b * RB;
    const double* rq = p.recQ + (size_t)b * RQ;
    const double d[3] = {xa[0] - __ldg(rb + B_X0), xa[1] - __ldg(rb + B_X1), xa[2] - __ldg(rb + B_X2)};
    const double mf = __ldg(rb + B_M) * fg;
    double gm[D];
#pragma unroll
    for (int k = 0; k < D; k++) gm[k] = mf * d[k];
    if (D == 3 && p.nbr_fe) gm[D - 1] = (__ldg(rb + B_M) * p.nbr_fe[(size_t)kk * n + i]) * d[D - 1];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const double q0 = __ldg(rq + c), al = __ldg(rq + 3 + c);
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        SQ0[c][k] += q0 * gm[k];
        SA[c][k] += al * gm[k];
        acc += __ldg(rq + 6 + 3 * k + c) * gm[k];
      }
      SQI[c] += acc;
    }
#pragma unroll
    for (int k = 0; k < D; k++) S1[k] += gm[k];
  }
  const double sla = p.slab[i];
  const double* rqA = p.recQ + (size_t)i * RQ;
  const double va[3] = {rbA[B_V0], rbA[B_V0 + 1], rbA[B_V0 + 2]};
  double vS1 = 0.0;
#pragma unroll
  for (int k = 0; k < D; k++) vS1 += va[k] * S1[k];
  double* df = p.dif;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double vq = 0.0, qs = 0.0;
#pragma unroll
    for (int k = 0; k < D; k++) {
      vq += va[k] * SQ0[c][k];
      qs += rqA[6 + 3 * k + c] * S1[k];
    }
    df[(size_t)(F_GQ + c) * n + i] = sla * (vq + rqA[c] * vS1);
    df[(size_t)(F_DQ + c) * n + i] = sla * (SQI[c] + qs);
#pragma unroll
    for (int k = 0; k < 3; k++)
      df[(size_t)(F_GA + 3 * k + c) * n + i] = (k < D) ? (SA[c][k] - rqA[3 + c] * S1[k]) / sla : 0.0;
  }
}

// ---------------------------------------------------------------------------
// pass B
// ---------------------------------------------------------------------------
// The 2-D launch is held to 168 registers (3 blocks, 12 warps an SM instead of
// 8): its loop and equations of motion are bound by the FP64 pipe, which more
// warps keep busier, at the cost of a few hundred bytes of spills (the FP64
// step 3.04 -> 2.94 ms at 160k particles; 128 registers was no better). The
// 3-D instantiations, with larger live sets, keep the plain bound.
template <int D, bool DIFF>
__global__ void __launch_bounds__(kBlock, (D == 2) ? 3 : 1) k_passB(RunConst rc, Ptrs p, int mode, double dt_sub) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double t = p.clock->t;
  const bool shear = rc.cfg.using_shear;
  const double* rbA = p.recB + (size_t)i * RB;
  const double xa[3] = {rbA[B_X0], rbA[B_X1], rbA[B_X2]};
  // separable accumulators: S1 = sum m grad W, SX = sum m X_b grad W, ...
  double S1[D], SP[D], SE[D], SB[D], SV[D][D], S0[D][D], SD[D];
#pragma unroll
  for (int k = 0; k < D; k++) {
    S1[k] = SP[k] = SE[k] = SB[k] = SD[k] = 0.0;
#pragma unroll
    for (int l = 0; l < D; l++) SV[k][l] = S0[k][l] = 0.0;
  }
  // the neighbours and grad-W factors pass A listed for this substep
  const int cnt = min(p.btrack[i], p.K);
  for (int kk = 0; kk < cnt; kk++) {
    const int b = p.nbr_idx[(size_t)kk * n + i];
    const double fg = p.nbr_f[(size_t)kk * n + i];
    const double* rb = p.recB + (size_t)b * RB;
    const double2 b01 = __ldg(reinterpret_cast<const double2*>(rb));
    const double2 b23 = __ldg(reinterpret_cast<const double2*>(rb + 2));
    double d[3] = {xa[0] - b01.x, xa[1] - b01.y, xa[2] - b23.x};
    {
      // grad_a W(r_a - r_b) = fg * d, reference src/kernel.cpp:95-118
      const double mf = b23.y * fg;   // m_b * (grad W)/rel
      double gm[D];
#pragma unroll
      for (int k = 0; k < D; k++) gm[k] = mf * d[k];
      if (D == 3 && p.nbr_fe) gm[D - 1] = (b23.y * p.nbr_fe[(size_t)kk * n + i]) * d[D - 1];   // factorised kernel
      const double2 b45 = __ldg(reinterpret_cast<const double2*>(rb + 4));
      const double2 b67 = __ldg(reinterpret_cast<const double2*>(rb + 6));
      const double2 v01 = __ldg(reinterpret_cast<const double2*>(rb + B_V0));
      const double vb[3] = {v01.x, v01.y, D == 3 ? __ldg(rb + B_V0 + 2) : 0.0};
#pragma unroll
      for (int k = 0; k < D; k++) {
        S1[k] += gm[k];
        SP[k] += b45.x * gm[k];
        SE[k] += b45.y * gm[k];
        SB[k] += b67.x * gm[k];
#pragma unroll
        for (int l = 0; l < D; l++) SV[k][l] += vb[l] * gm[k];
      }
      if (shear) {
        double p0[3], pij[6];
#pragma unroll
        for (int k = 0; k < D; k++) p0[k] = __ldg(rb + B_PI0 + k);
#pragma unroll
        for (int k = 0; k < 6; k++) pij[k] = (D == 3 || (k != 2 && k != 4 && k != 5)) ? __ldg(rb + B_PIJ + k) : 0.0;
        // pi^{ij}/sl^2 with (11 12 13 22 23 33) packing
        auto PJ = [&](int a_, int b_) {
          const int lo = a_ < b_ ? a_ : b_, hi = a_ < b_ ? b_ : a_;
          return pij[lo == 0 ? hi : (lo == 1 ? 2 + hi : 5)];
        };
#pragma unroll
        for (int k = 0; k < D; k++) {
#pragma unroll
          for (int l = 0; l < D; l++) S0[k][l] += p0[l] * gm[k];
          // one FMA a term into the sum (the FP64 pipe bounds this loop)
#pragma unroll
          for (int l = 0; l < D; l++) SD[k] = fma(PJ(k, l), gm[l], SD[k]);
        }
      }
    }
  }
  // own values
  const double sla = p.slab[i];
  const double ea = rbA[B_E], Pa = rbA[B_P], Pia = rbA[B_PI];
  double va[3] = {rbA[B_V0], rbA[B_V0 + 1], D == 3 ? rbA[B_V0 + 2] : 0.0};
  double gP[3] = {0, 0, 0}, gE[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gS[3] = {0, 0, 0}, dS[3] = {0, 0, 0};
  double gV[9] = {0};
  double vS1 = 0.0;
#pragma unroll
  for (int k = 0; k < D; k++) vS1 += va[k] * S1[k];
#pragma unroll
  for (int k = 0; k < D; k++) {
    gP[k] = sla * (SP[k] + Pa * S1[k]);
    gE[k] = (SE[k] - ea * S1[k]) / sla;
    gB[k] = sla * (SB[k] + Pia * S1[k]);
#pragma unroll
    for (int l = 0; l < D; l++) gV[k * D + l] = (SV[k][l] - va[l] * S1[k]) / sla;
    if (shear) {
      double acc = 0.0;
#pragma unroll
      for (int l = 0; l < D; l++) acc += va[l] * S0[l][k];
      gS[k] = sla * (acc + rbA[B_PI0 + k] * vS1);
      double acc2 = SD[k];
#pragma unroll
      for (int l = 0; l < D; l++) {
        const int lo = k < l ? k : l, hi = k < l ? l : k;
        acc2 += rbA[B_PIJ + (lo == 0 ? hi : (lo == 1 ? 2 + hi : 5))] * S1[l];
      }
      dS[k] = sla * acc2;
    }
  }
  finish_particle<D, double, false, DIFF>(rc, p, i, mode, t, dt_sub, va, gP, gE, gB, gS, dS, gV);
}

__global__ void k_visc(RunConst rc, Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  double th[NTH];
  for (int q = 0; q < NTH; q++) th[q] = p.th[q * n + i];
  const Transport k = transport(rc.cfg, th);
  p.derivs[D_ETA * n + i] = k.eta;
  p.derivs[D_TAUPI * n + i] = k.tau_pi;
  p.derivs[D_ZETA * n + i] = k.zeta;
  p.derivs[D_TAUBULK * n + i] = k.tau_Pi;
}

__global__ void k_clock(Clock* c, int substep, double dt) { advance_clock(c, substep, dt); }

// ---------------------------------------------------------------------------
// initialisation (reference src/sph_workstation.cpp:252-375, :1228-1340)
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_init_state(RunConst rc, Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double t = rc.cfg.coord == 1 ? 1.0 : p.clock->t;   // the metric's tau (1 in Cartesian coordinates)
  const double u3[3] = {p.y[Y_U0 * n + i], p.y[Y_U1 * n + i], D == 3 ? p.y[Y_U2 * n + i] : 0.0};
  const double g = gamma_milne<D>(u3, t * t);
  p.gam[i] = g;
  for (int q = 0; q < 3; q++) p.v[q * n + i] = (q < D) ? u3[q] / g : 0.0;
  p.m[i] = 1.0;
  for (int q = Y_ES; q <= Y_EQ; q++) p.y[q * n + i] = 1.0;
  p.y[Y_EBULK * n + i] = 0.0;
  for (int q = 0; q < 5; q++) p.y[(Y_SHV0 + q) * n + i] = 0.0;
  p.y[Y_EZ * n + i] = 0.0;
  p.th[T_T * n + i] = 580.0 / kHbarcMeVfm;
  p.th[T_MUB * n + i] = p.th[T_MUS * n + i] = p.th[T_MUQ * n + i] = 0.0;
  p.eos_id[i] = 0;
  p.freeze[i] = 0;
  double2* ra = reinterpret_cast<double2*>(p.recA) + (size_t)i * 4;
  ra[0] = make_double2(p.y[Y_X0 * n + i], p.y[Y_X1 * n + i]);
  ra[1] = make_double2(D == 3 ? p.y[Y_X2 * n + i] : 0.0, 1.0);
  p.posf[i] = make_float4((float)p.y[Y_X0 * n + i], (float)p.y[Y_X1 * n + i],
                          D == 3 ? (float)p.y[Y_X2 * n + i] : 0.0f, 0.0f);
  ra[2] = make_double2(1.0, 1.0);
  ra[3] = make_double2(1.0, 1.0);
}

// ext = input/sigma after the initial sigma (src/sph_workstation.cpp:338-364)
template <int D>
__global__ void k_init_ext(RunConst rc, Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double sg = p.sig[i];
  const double es = p.in_s[i] / sg;
  p.y[Y_ES * n + i] = es;
  p.y[Y_EB * n + i] = p.in_rho[i] / sg;
  p.y[Y_ESS * n + i] = p.in_rho[n + i] / sg;
  p.y[Y_EQ * n + i] = p.in_rho[2 * n + i] / sg;
  if (p.in_s[i] < 0.0) p.freeze[i] = 4;
  const double m = p.m[i];
  double2* ra = reinterpret_cast<double2*>(p.recA) + (size_t)i * 4;
  ra[2] = make_double2(m * es, m * p.y[Y_EB * n + i]);
  ra[3] = make_double2(m * p.y[Y_ESS * n + i], m * p.y[Y_EQ * n + i]);
}

// Initial viscous state (src/sph_workstation.cpp:1350-1430): with
// bulk_from_trace, ext Pi = (trace - p) / sigma (p of the e -> s inversion);
// with input_initial_shear, ext pi^{ij} = pi^{ij} / sigma for (1,1) (1,2)
// (1,3) (2,2) (2,3). iv: the input trace, then pi^{xx xy xeta yy yeta}.
__global__ void k_init_viscous(Ptrs p, const double* iv, int bulk, int shear) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double sg = p.sig[i];
  if (bulk) p.y[Y_EBULK * n + i] = (iv[i] - p.th[T_P * n + i]) / sg;
  if (shear)
#pragma unroll
    for (int k = 0; k < 5; k++) p.y[(Y_SHV0 + k) * n + i] = iv[(size_t)(1 + k) * n + i] / sg;
}

// set_diffusion (src/sph_workstation.cpp:1441-1458): ext q = q^i / sigma;
// iq: the initial spatial currents q^i (3c + i), or null for none
__global__ void k_init_diffusion(Ptrs p, const double* iq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double sg = p.sig[i];
#pragma unroll
  for (int q = 0; q < 9; q++) p.dif[(size_t)(F_YQ + q) * n + i] = iq ? iq[(size_t)q * n + i] / sg : 0.0;
}

// FP64 smoothing record from the state (after mixed substeps moved the particles)
template <int D>
__global__ void k_pack_fp64(Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double x[3] = {p.y[Y_X0 * n + i], p.y[Y_X1 * n + i], D == 3 ? p.y[Y_X2 * n + i] : 0.0};
  const double ext[4] = {p.y[Y_ES * n + i], p.y[Y_EB * n + i], p.y[Y_ESS * n + i], p.y[Y_EQ * n + i]};
  write_recA<D>(p, i, x, p.m[i], ext);
}

// ---------------------------------------------------------------------------
// conservation sums (src/system_state.cpp:738-885): per-block partials in a
// fixed order, summed on the host
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_totals(RunConst rc, Ptrs p) {
  __shared__ double sh[6][256];
  const int n = p.n;
  const double t = p.clock->t;
  const double sqrtg = rc.cfg.coord == 0 ? t : 1.0;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double m = p.m[i];
    const double g = p.gam[i];
    acc[0] += p.y[Y_ES * n + i] * m;
    if (p.dif) {
      // the q^0 terms of src/system_state.cpp:755-828, with the reference's
      // mass factors
      const double sg = p.sig[i];
      const double eqb = p.dif[(size_t)F_Q * n + i] * m / sg / g;
      const double eqs = p.dif[(size_t)(F_Q + 4) * n + i] * m / sg / g;
      const double eqq = p.dif[(size_t)(F_Q + 8) * n + i] * m / sg / g;
      acc[1] += p.y[Y_EB * n + i] * m + eqb * m / g;
      acc[2] += p.y[Y_ESS * n + i] * m + (eqs);
      acc[3] += p.y[Y_EQ * n + i] * m + (eqq);
    } else {
      acc[1] += p.y[Y_EB * n + i] * m;
      acc[2] += p.y[Y_ESS * n + i] * m;
      acc[3] += p.y[Y_EQ * n + i] * m;
    }
    const double C = p.th[T_W * n + i] + p.bulk[i];
    acc[4] += (C * g * g - p.th[T_P * n + i] - p.bulk[i] + p.pi[P00 * n + i]) * m * sqrtg / p.slab[i];
    acc[5] += p.y[Y_EZ * n + i];
  }
  for (int q = 0; q < 6; q++) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int q = 0; q < 6; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 6; q++) p.partials[blockIdx.x * 6 + q] = sh[q][0];
}

// ---------------------------------------------------------------------------
// explicit neighbour list (parity checks only)
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_nbr_count(RunConst rc, Ptrs p, int32_t* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double xa[3] = {p.y[Y_X0 * p.n + i], p.y[Y_X1 * p.n + i], D == 3 ? p.y[Y_X2 * p.n + i] : 0.0};
  int c = 0;
  for_candidates<D>(rc, p, i, xa, [&](int b) {
    double d[3] = {xa[0] - p.y[Y_X0 * p.n + b], xa[1] - p.y[Y_X1 * p.n + b],
                   D == 3 ? xa[2] - p.y[Y_X2 * p.n + b] : 0.0};
    if (dist2_exact<D>(d) <= rc.cut2) c++;
  });
  counts[i] = c;
}

template <int D>
__global__ void k_nbr_fill(RunConst rc, Ptrs p, const int32_t* off, int32_t* idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double xa[3] = {p.y[Y_X0 * p.n + i], p.y[Y_X1 * p.n + i], D == 3 ? p.y[Y_X2 * p.n + i] : 0.0};
  int c = off[i];
  for_candidates<D>(rc, p, i, xa, [&](int b) {
    double d[3] = {xa[0] - p.y[Y_X0 * p.n + b], xa[1] - p.y[Y_X1 * p.n + b],
                   D == 3 ? xa[2] - p.y[Y_X2 * p.n + b] : 0.0};
    if (dist2_exact<D>(d) <= rc.cut2) idx[c++] = b;
  });
}

// One block: the largest T and the number of frozen particles, tau and the
// error counters.
__global__ void __launch_bounds__(1024) k_probe(Ptrs p, Probe* out) {
  __shared__ double red[32];
  __shared__ int32_t redc[32];
  double m = 0.0;
  int32_t c = 0;
  const double* T = p.th + T_T * p.n;
  for (int i = threadIdx.x; i < p.n; i += blockDim.x) {
    m = fmax(m, T[i]);
    c += p.freeze[i] >= 4 ? 1 : 0;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5] = m;
    redc[threadIdx.x >> 5] = c;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool in = threadIdx.x < (blockDim.x >> 5);
    m = in ? red[threadIdx.x] : 0.0;
    c = in ? redc[threadIdx.x] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (threadIdx.x == 0) {
      out->maxT = m;
      out->tau = p.clock->t;
      for (int q = 0; q < NERR; q++) out->err[q] = p.err[q];
      out->frozen = c;
    }
  }
}

// Freeze-out status machine after a step (reference include/freeze_out.h:
// check_freeze_out_status :455-500, then bsqsvfreezeout :549-615 without the
// hypersurface output): 0 -> 1 when e <= e_FO; 1 -> 3 when the particle lost
// its neighbours or e stayed <= e_FO without rising, 1 -> 1 when e rose, else
// back to 0; from the third step on, particles without neighbours freeze
// (freeze_out_evo :322-375), status 3 becomes 4 (:914) and the energy of
// the live particles is snapshotted.
__global__ void k_freeze(RunConst rc, Ptrs p) { freeze_particle(rc, p, blockIdx.x * blockDim.x + threadIdx.x); }

// The freeze-out stage with the hypersurface (cfg.surface), after a step:
// check_freeze_out_status (include/freeze_out.h:455-500) and bsqsvfreezeout
// (:549-615) per particle. Snapshots of every field (first step: frz2;
// second: frz1; later: the few-neighbour backups and restores of
// freeze_out_evo, :322-375, the no-neighbour freeze, the interpolation, then
// frz2 <- frz1 for the live particles and frz1 <- now for all). A particle at
// status 3 is interpolated (bsqsvinterpolate, :617-936) from the snapshot
// whose energy is closer to e_FO, its freeze_out.dat row appended
// (src/output.cpp:433-475; the order of the appends is fixed on the host),
// and it becomes 4. The current gradients, theta and shv_nabla_u are those
// of the last derivative evaluation (recomputed before this kernel).
template <int D>
__global__ void k_freeze_surface(RunConst rc, Ptrs p, int grads_f32, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const Clock c = *p.clock;
  const int frzc = c.frzc;
  const double ef = rc.efreeze, t = c.t;
  const double taup = frzc == 1 ? t : c.taup, taupp = c.taupp;
  auto SN = [&](int k, int q) -> double& { return p.fz[((size_t)k * NSF + q) * n + i]; };
  auto copy_snap = [&](int dst, int src) {
    for (int q = 0; q < NSF; q++) SN(dst, q) = SN(src, q);
  };
  const float* gf = reinterpret_cast<const float*>(p.grads);
  auto G = [&](int slot) { return grads_f32 ? double(gf[(size_t)slot * n + i]) : p.grads[(size_t)slot * n + i]; };
  // the current values
  double cur[NSF];
  for (int k = 0; k < 3; k++) {
    cur[SF_R + k] = k < D ? p.y[(Y_X0 + k) * n + i] : 0.0;
    cur[SF_U + k] = k < D ? p.y[(Y_U0 + k) * n + i] : 0.0;
    cur[SF_GP + k] = k < D ? G(G_P + k) : 0.0;
    cur[SF_GE + k] = k < D ? G(G_E + k) : 0.0;
  }
  cur[SF_S] = p.th[T_S * n + i];
  cur[SF_E] = p.th[T_E * n + i];
  cur[SF_RB] = p.th[T_RB * n + i];
  cur[SF_RS] = p.th[T_RS * n + i];
  cur[SF_RQ] = p.th[T_RQ * n + i];
  cur[SF_T] = p.th[T_T * n + i];
  cur[SF_MUB] = p.th[T_MUB * n + i];
  cur[SF_MUS] = p.th[T_MUS * n + i];
  cur[SF_MUQ] = p.th[T_MUQ * n + i];
  cur[SF_THETA] = p.derivs[D_THETA * n + i];
  cur[SF_BULK] = p.bulk[i];
  cur[SF_SLAB] = p.slab[i];
  const int sl[10][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {1, 1}, {1, 2}, {1, 3}, {2, 2}, {2, 3}, {3, 3}};
  for (int q = 0; q < 10; q++) cur[SF_SHV + q] = p.pi[pi_slot(sl[q][0], sl[q][1]) * n + i];
  cur[SF_SHV33] = p.pi[pi_slot(3, 3) * n + i];
  cur[SF_SNU] = p.derivs[D_SNU * n + i];
  cur[SF_W] = p.th[T_W * n + i];
  cur[SF_CS2] = p.th[T_CS2 * n + i];
  // the diffusion current q^mu of the evaluation (zero without the sector)
  for (int k = 0; k < 12; k++) cur[SF_Q + k] = p.dif ? p.dif[(size_t)(F_Q + k) * n + i] : 0.0;
  // check_freeze_out_status
  int f = p.freeze[i];
  const double e = cur[SF_E];
  if (f == 0) {
    if (e <= ef) f = 1;
  } else if (f == 1) {
    if (p.btrack[i] == -1) f = 3;
    else if (e > p.frz1_e[i]) f = 1;
    else if (e <= ef) f = 3;
    else f = 0;
  }
  // bsqsvinterpolate from snapshot k taken at tp
  auto interpolate = [&](int k, double tp) {
    const double tlist = p.btrack[i] != -1 ? tp : tp - dt;
    const double t2 = tlist * tlist;
    double uout[3], ucov[3], gP[3], gE[3], gPc[3], gEc[3];
    for (int a = 0; a < D; a++) {
      uout[a] = SN(k, SF_U + a);
      gP[a] = SN(k, SF_GP + a);
      gE[a] = SN(k, SF_GE + a);
      ucov[a] = -uout[a];
      gPc[a] = -gP[a];
      gEc[a] = -gE[a];
    }
    if (rc.cfg.coord == 0 && D == 3) {
      ucov[2] = uout[2] * -t2;
      gPc[2] = gP[2] * (-1. / t2);
      gEc[2] = gE[2] * (-1. / t2);
    }
    const double bulk = SN(k, SF_BULK), theta = SN(k, SF_THETA), snu = SN(k, SF_SNU);
    double sigsub = SN(k, SF_SLAB);
    double Tfluc = SN(k, SF_T), sFO = SN(k, SF_S);
    double norm2 = 0.0;
    for (int a = 0; a < D; a++) norm2 += uout[a] * ucov[a];
    const double gsub = sqrt(-norm2 + 1);
    if (rc.cfg.coord == 1) sigsub /= gsub;
    else sigsub /= gsub * tlist;
    const double swsub = p.m[i] / sigsub;
    double divT[3], divE[3], divTc[3];
    for (int a = 0; a < D; a++) {
      divT[a] = (1.0 / sFO) * gP[a];
      divE[a] = gE[a];
      divTc[a] = (1.0 / sFO) * gPc[a];
    }
    const double cs2 = SN(k, SF_CS2), w = SN(k, SF_W);
    double inner = 0;
    for (int a = 0; a < D; a++) inner += uout[a] * gP[a];
    const double divPpress = -(1.0 / gsub) * (cs2 * (w + bulk) * theta - cs2 * snu + inner);
    double divTtemp = divPpress / sFO;
    inner = 0;
    for (int a = 0; a < D; a++) inner += uout[a] * gE[a];
    double divEener = -(1.0 / gsub) * ((w + bulk) * theta - snu + inner);
    norm2 = 0;
    for (int a = 0; a < D; a++) norm2 += divT[a] * divTc[a];
    double nrm = -sqrt(fabs(divTtemp * divTtemp + norm2));
    nrm = fabs(nrm) > 1.E-14 ? nrm : 1.E-14;
    divTtemp /= nrm;
    for (int a = 0; a < D; a++) divT[a] /= nrm;
    norm2 = 0;
    for (int a = 0; a < D; a++) norm2 += divE[a] * gEc[a];
    double nrmE = -sqrt(fabs(divEener * divEener + norm2));
    nrmE = fabs(nrmE) > 1.E-14 ? nrmE : 1.E-14;
    divEener /= nrmE;
    for (int a = 0; a < D; a++) divE[a] /= nrmE;
    sFO *= pow(Tfluc * kHbarcGeVfm, 3);
    Tfluc *= kHbarcGeVfm;
    const int row = atomicAdd(p.fo_count, 1);
    if (row >= n) return;   // never: a particle is interpolated once
    double* r = p.fo_rows + (size_t)row * kFoRow;
    int w_ = 0;
    r[w_++] = (double)c.nstep;
    r[w_++] = (double)i;
    r[w_++] = divEener;
    for (int a = 0; a < D; a++) r[w_++] = divE[a];
    r[w_++] = gsub;
    for (int a = 0; a < D; a++) r[w_++] = uout[a];
    r[w_++] = swsub;
    r[w_++] = bulk;
    r[w_++] = SN(k, SF_SHV + 0);
    r[w_++] = SN(k, SF_SHV + 4);
    r[w_++] = SN(k, SF_SHV + 7);
    r[w_++] = SN(k, SF_SHV33);
    r[w_++] = SN(k, SF_SHV + 5);
    if (D != 2) {
      r[w_++] = SN(k, SF_SHV + 6);
      r[w_++] = SN(k, SF_SHV + 8);
    }
    r[w_++] = tlist;
    for (int a = 0; a < D; a++) r[w_++] = SN(k, SF_R + a);
    const double tail[11] = {sFO, SN(k, SF_E), Tfluc, SN(k, SF_MUB), SN(k, SF_MUS), SN(k, SF_MUQ), w, cs2,
                             SN(k, SF_RB), SN(k, SF_RS), SN(k, SF_RQ)};
    for (int a = 0; a < 11; a++) r[w_++] = tail[a];
    for (int a = 0; a < 12; a++) r[w_++] = SN(k, SF_Q + a);   // q^mu of the snapshot (diffout)
    r[w_++] = (rc.cfg.eos_kind == 2 && p.eos_id[i] == 0) ? 1.0 : 0.0;
  };
  auto closer = [&]() { return fabs(SN(0, SF_E) - ef) < fabs(SN(1, SF_E) - ef) ? 0 : 1; };
  if (frzc == 0) {
    for (int q = 0; q < NSF; q++) SN(1, q) = cur[q];
  } else if (frzc == 1) {
    p.frz1_e[i] = e;
    for (int q = 0; q < NSF; q++) SN(0, q) = cur[q];
    if (f == 3) {
      const int k = closer();
      interpolate(k, k == 0 ? taup : taupp);
      f = 4;
    }
  } else {
    const int bt = p.btrack[i];
    if (f < 4 && bt <= 3 && bt > 0) {
      copy_snap(5, 3);
      copy_snap(4, 2);
      copy_snap(3, 1);
      copy_snap(2, 0);
    }
    if (f < 4 && bt == 0 && SN(2, SF_GP) != 0) {
      copy_snap(1, 3);
      copy_snap(0, 2);
    }
    if (f < 4 && bt == 0 && SN(2, SF_GP) == 0) {
      copy_snap(1, 5);
      copy_snap(0, 4);
    }
    if (f < 4 && bt == 0) {
      f = 4;
      p.btrack[i] = -1;
    }
    if (f == 3) {
      const int k = closer();
      interpolate(k, k == 0 ? taup : taupp);
      f = 4;
    }
    if (f < 4) copy_snap(1, 0);
    for (int q = 0; q < NSF; q++) SN(0, q) = cur[q];
    if (f < 4) p.frz1_e[i] = e;
  }
  p.freeze[i] = f;
}

__global__ void k_freeze_surface_advance(Clock* c) {
  if (c->frzc == 0) c->taupp = c->t;
  else if (c->frzc == 1) c->taup = c->t;
  else {
    c->taupp = c->taup;
    c->taup = c->t;
  }
  if (c->frzc < 2) c->frzc++;
  c->nstep++;
}

__global__ void k_freeze_advance(Clock* c) {
  if (c->frzc < 2) c->frzc++;
}

// Diagnostics of the last derivative evaluation (the substep-2 evaluation of
// the last RK2 step, at t = t0 + dt/2), for the system-state output: the
// equations of motion again from the stored inputs of that evaluation
// (thermodynamics, gradients, pi^{mu nu}, Pi, gamma, v; u = gamma v), with
// theta and sigma^{ij} taken out (src/eom_default.cpp:774-807), the transport
// coefficients, and, with shear, src/eom_default.cpp:1831-1985
// (compute_hydro_numbers): sigma^{mu nu} completed by symmetry,
// orthogonality to u and tracelessness, Knudsen numbers tau_pi
// sqrt|sigma:sigma| and tau_Pi |theta|, inverse Reynolds numbers
// sqrt|pi:pi| / p and |Pi| / p. grads_f32: the gradients are the mixed
// form's FP32 view.
template <int D, bool DIFF>
__global__ void k_diag(RunConst rc, Ptrs p, int grads_f32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double t = p.clock->teval;
  const double t2 = rc.cfg.coord == 1 ? 1.0 : t * t;
  double th[NTH];
#pragma unroll
  for (int q = 0; q < NTH; q++) th[q] = p.th[q * n + i];
  const float* gf = reinterpret_cast<const float*>(p.grads);
  auto G = [&](int slot) { return grads_f32 ? double(gf[(size_t)slot * n + i]) : p.grads[(size_t)slot * n + i]; };
  EomIn<D, double> in;
  in.th = th;
  in.it = 1.0 / t;
  in.it2 = 1.0 / (t * t);
  in.g = p.gam[i];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    in.v[q] = p.v[q * n + i];
    in.u[q] = (q < D) ? in.v[q] * in.g : 0.0;
    in.gradP[q] = (q < D) ? G(G_P + q) : 0.0;
    in.gradBulk[q] = (q < D) ? G(G_B + q) : 0.0;
    in.gradshear[q] = (q < D) ? G(G_SH + q) : 0.0;
    in.divshear[q] = (q < D) ? G(G_DS + q) : 0.0;
  }
#pragma unroll
  for (int q = 0; q < 9; q++) in.gradV[q] = (q < D * D) ? G(G_V + q) : 0.0;
  in.sigma = p.sig[i];
  in.sigma_lab = p.slab[i];
  in.m = p.m[i];
  in.Pi = p.bulk[i];
#pragma unroll
  for (int q = 0; q < NPI; q++) in.pi[q] = p.pi[q * n + i];
  const TransportT<double> k = transport<double>(rc.cfg, th);
  EomOut<double> o;
  double dg[7];
  if constexpr (DIFF) {
    // with the diffusion sector: its coupling into du/dt, and its Knudsen
    // and inverse Reynolds numbers (src/eom_default.cpp:1944-1982)
    DiffIn din;
    DiffOut dout;
    load_diff_in(rc, p, i, th, din);
    eom<D, double>(rc.cfg, k, in, t, o, dg, &din, &dout);
    const double rho[3] = {th[T_RB], th[T_RS], th[T_RQ]};
    for (int c = 0; c < 3; c++) {
      double gsq = 0.0;
      for (int a = 0; a < D; a++) {
        const double gg = din.ga[3 * a + c];
        gsq += gg * gg;
      }
      p.dif[(size_t)(F_KN + c) * n + i] = din.tq[4 * c] * sqrt(gsq);
      const double* q = din.q + 4 * c;
      const double q_sq = q[1] * q[1] + q[2] * q[2] + t2 * q[3] * q[3] - q[0] * q[0];
      const double q_mag = q_sq > 0.0 ? sqrt(q_sq) : 0.0;
      const double n_abs = fabs(rho[c]);
      p.dif[(size_t)(F_IR + c) * n + i] = (n_abs > 1e-15) ? q_mag / n_abs : 0.0;
    }
  } else {
    eom<D, double>(rc.cfg, k, in, t, o, dg);
  }
  double* dv = p.derivs;
  dv[D_ETA * n + i] = k.eta;
  dv[D_TAUPI * n + i] = k.tau_pi;
  dv[D_ZETA * n + i] = k.zeta;
  dv[D_TAUBULK * n + i] = k.tau_Pi;
  dv[D_THETA * n + i] = dg[0];
  dv[D_SNU * n + i] = dg[6];
  double kns = 0.0, knb = 0.0, irs = 0.0, irb = 0.0;
  // computed with shear or diffusion (src/eom_default.cpp:865-867); without
  // shear the sigma tensor and pi are zero
  if (rc.cfg.using_shear || DIFF) {
    for (int q = 0; q < 5; q++) dv[(D_SIG0 + q) * n + i] = dg[1 + q];
    const double g = in.g;
    const double uc[3] = {-in.u[0], -in.u[1], D == 3 ? -t2 * in.u[2] : 0.0};
    double st[4][4];
    for (int a = 0; a < 4; a++) for (int b = 0; b < 4; b++) st[a][b] = 0.0;
    st[1][1] = dg[1]; st[1][2] = dg[2]; st[1][3] = dg[3]; st[2][2] = dg[4]; st[2][3] = dg[5];
    for (int a = 1; a < 4; a++) for (int b = a + 1; b < 4; b++) st[b][a] = st[a][b];
    for (int a = 1; a < D + 1; a++) {
      double c = 0.0;
      for (int b = 1; b < D + 1; b++) c += uc[b - 1] * st[a][b];
      st[0][a] = -1. * c / g;
    }
    for (int a = 1; a < 4; a++) st[a][0] = st[0][a];
    st[0][0] = (uc[0] * uc[0] * st[1][1] + uc[1] * uc[1] * st[2][2] + 2. * uc[1] * uc[0] * st[2][1] +
                2. * uc[2] * uc[0] * st[3][1] + 2. * uc[2] * uc[1] * st[3][2] -
                uc[2] * uc[2] * (st[1][1] + st[2][2]) / t2) /
               (g * g - uc[2] * uc[2] / t2);
    st[3][3] = (st[0][0] - st[1][1] - st[2][2]) / t2;
    const double gm[4] = {1.0, -1.0, -1.0, -t2};
    double sn = 0.0, pn = 0.0;
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++) {
        sn += st[a][b] * (st[a][b] * gm[b] * gm[a]);
        const double pab = in.pi[pi_slot(a, b)];
        pn += pab * (pab * gm[b] * gm[a]);
      }
    const double pr = th[T_P];
    kns = k.tau_pi * sqrt(fabs(sn));
    knb = k.tau_Pi * fabs(dg[0]);
    irs = sqrt(fabs(pn)) / pr;
    irb = fabs(in.Pi) / pr;
  } else {
    for (int q = 0; q < 5; q++) dv[(D_SIG0 + q) * n + i] = 0.0;
  }
  dv[D_KNS * n + i] = kns;
  dv[D_KNB * n + i] = knb;
  dv[D_IRS * n + i] = irs;
  dv[D_IRB * n + i] = irb;
}

// FP32 copy of the table densities (fields 1..5 of 17) at 8 floats a node.
__global__ void k_table_f32(const double* f, float* fd, int64_t nodes) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nodes) return;
  const double* node = f + q * 17;
  float4* o = reinterpret_cast<float4*>(fd + q * 8);
  o[0] = make_float4((float)node[1], (float)node[2], (float)node[3], (float)node[4]);
  o[1] = make_float4((float)node[5], 0.0f, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(1024) k_count_frozen(Ptrs p, int32_t* out) {
  __shared__ int32_t red[32];
  int32_t c = 0;
  for (int i = threadIdx.x; i < p.n; i += blockDim.x) c += p.freeze[i] >= 4 ? 1 : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    c = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) *out = c;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_build_cells(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  cudaMemsetAsync(p.cell_count, 0, sizeof(int32_t) * rc.grid.ncell, s);
  if (rc.cfg.dim == 3) k_bin<3><<<nb, kBlock, 0, s>>>(rc, p);
  else k_bin<2><<<nb, kBlock, 0, s>>>(rc, p);
  const int ncell = rc.grid.ncell;
  const int ntiles = scan_tiles(ncell);
  k_scan_tiles<<<ntiles, kScanThreads, 0, s>>>(p.cell_count, p.cell_start, p.scan_aux, ncell);
  k_scan_add<<<(ncell + 255) / 256, 256, 0, s>>>(p.cell_start, p.scan_aux, ncell, ntiles);
  k_scatter<<<nb, kBlock, 0, s>>>(p);
  k_sort_cells<<<(int)(((int64_t)ncell * 32 + 255) / 256), 256, 0, s>>>(p, ncell);
}

void launch_candidates(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_candidates<3><<<nb, kBlock, 0, s>>>(rc, p);
  else k_candidates<2><<<nb, kBlock, 0, s>>>(rc, p);
}

void launch_passA(const RunConst& rc, const EosDev& eos, const Ptrs& p, int mode, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_passA<3><<<nb, kBlock, 0, s>>>(rc, p);
  else k_passA<2><<<nb, kBlock, 0, s>>>(rc, p);
  if (mode == A_WITH_THERMO) launch_thermo(rc, eos, p, s);
}

// With the diffusion sector, its gradient sums run first (they read the
// diffusion records of the neighbours, complete after the thermo pass).
void launch_passB(const RunConst& rc, const Ptrs& p, int mode, double dt_sub, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  const bool dif = rc.cfg.using_diffusion && p.dif;
  if (rc.cfg.dim == 3) {
    if (dif) {
      k_diffgrad<3><<<nb, kBlock, 0, s>>>(p);
      k_passB<3, true><<<nb, kBlock, 0, s>>>(rc, p, mode, dt_sub);
    } else {
      k_passB<3, false><<<nb, kBlock, 0, s>>>(rc, p, mode, dt_sub);
    }
  } else {
    if (dif) {
      k_diffgrad<2><<<nb, kBlock, 0, s>>>(p);
      k_passB<2, true><<<nb, kBlock, 0, s>>>(rc, p, mode, dt_sub);
    } else {
      k_passB<2, false><<<nb, kBlock, 0, s>>>(rc, p, mode, dt_sub);
    }
  }
}

void launch_visc(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  k_visc<<<(p.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(rc, p);
}

void launch_clock(const Ptrs& p, int substep, double dt, cudaStream_t s) { k_clock<<<1, 1, 0, s>>>(p.clock, substep, dt); }

void launch_init_state(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_init_state<3><<<nb, kBlock, 0, s>>>(rc, p);
  else k_init_state<2><<<nb, kBlock, 0, s>>>(rc, p);
}

// The input densities as rows (e|s, rhoB, rhoS, rhoQ), for the seed network.
__global__ void k_pack_inputs(Ptrs p, double* in4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  in4[(size_t)4 * i] = p.in_e[i];
  for (int c = 0; c < 3; c++) in4[(size_t)4 * i + 1 + c] = p.in_rho[(size_t)c * n + i];
}

__global__ void k_sph_kernel(RunConst rc, int64_t n, const double* r2, double* w, double* fg) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d2 = r2[i];
  double W = 0.0, f = 0.0;
  if ((unsigned long long)__double_as_longlong(d2) <= rc.cut2_bits) pair_kernel_warp(rc, d2, W, f);
  w[i] = W;
  fg[i] = f;
}

void launch_sph_kernel(const RunConst& rc, int64_t n, const double* r2, double* w, double* fg, cudaStream_t s) {
  k_sph_kernel<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(rc, n, r2, w, fg);
}

void launch_pack_inputs(const Ptrs& p, double* in4, cudaStream_t s) {
  k_pack_inputs<<<(p.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(p, in4);
}

void launch_init_ext(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_init_ext<3><<<nb, kBlock, 0, s>>>(rc, p);
  else k_init_ext<2><<<nb, kBlock, 0, s>>>(rc, p);
}

void launch_init_viscous(const Ptrs& p, const double* iv, int bulk, int shear, cudaStream_t s) {
  if (iv && (bulk || shear)) k_init_viscous<<<(p.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(p, iv, bulk, shear);
}

void launch_init_diffusion(const Ptrs& p, const double* iq, cudaStream_t s) {
  if (p.dif) k_init_diffusion<<<(p.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(p, iq);
}

void launch_pack_fp64(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_pack_fp64<3><<<nb, kBlock, 0, s>>>(p);
  else k_pack_fp64<2><<<nb, kBlock, 0, s>>>(p);
}

void launch_probe(const Ptrs& p, Probe* out, cudaStream_t s) { k_probe<<<1, 1024, 0, s>>>(p, out); }

void launch_freeze(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  k_freeze<<<(p.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(rc, p);
  k_freeze_advance<<<1, 1, 0, s>>>(p.clock);
}

void launch_count_frozen(const Ptrs& p, int32_t* out, cudaStream_t s) { k_count_frozen<<<1, 1024, 0, s>>>(p, out); }

void launch_freeze_surface(const RunConst& rc, const Ptrs& p, int grads_f32, double dt, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_freeze_surface<3><<<nb, kBlock, 0, s>>>(rc, p, grads_f32, dt);
  else k_freeze_surface<2><<<nb, kBlock, 0, s>>>(rc, p, grads_f32, dt);
  k_freeze_surface_advance<<<1, 1, 0, s>>>(p.clock);
}

void launch_diagnostics(const RunConst& rc, const Ptrs& p, int grads_f32, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  const bool dif = rc.cfg.using_diffusion && p.dif;
  if (rc.cfg.dim == 3) {
    if (dif) k_diag<3, true><<<nb, kBlock, 0, s>>>(rc, p, grads_f32);
    else k_diag<3, false><<<nb, kBlock, 0, s>>>(rc, p, grads_f32);
  } else {
    if (dif) k_diag<2, true><<<nb, kBlock, 0, s>>>(rc, p, grads_f32);
    else k_diag<2, false><<<nb, kBlock, 0, s>>>(rc, p, grads_f32);
  }
}

void launch_table_f32(const double* f, float* fd, int64_t nodes, cudaStream_t s) {
  if (nodes <= 0) return;
  k_table_f32<<<(unsigned)((nodes + 255) / 256), 256, 0, s>>>(f, fd, nodes);
}

void launch_totals(const RunConst& rc, const Ptrs& p, int nblocks, cudaStream_t s) {
  k_totals<<<nblocks, 256, 0, s>>>(rc, p);
}

void launch_neighbour_counts(const RunConst& rc, const Ptrs& p, int32_t* counts, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_nbr_count<3><<<nb, kBlock, 0, s>>>(rc, p, counts);
  else k_nbr_count<2><<<nb, kBlock, 0, s>>>(rc, p, counts);
}

void launch_neighbour_fill(const RunConst& rc, const Ptrs& p, const int32_t* offsets, int32_t* idx, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_nbr_fill<3><<<nb, kBlock, 0, s>>>(rc, p, offsets, idx);
  else k_nbr_fill<2><<<nb, kBlock, 0, s>>>(rc, p, offsets, idx);
}

}  // namespace ccake
