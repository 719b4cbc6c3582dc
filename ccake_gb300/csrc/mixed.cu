// Mixed-precision form of the two fused passes (ccake_config.precision = 1).
//
// The pair loops run in FP32: positions travel as (hi, lo) float pairs, so a
// pair displacement (hi_a - hi_b) + (lo_a - lo_b) keeps FP32 precision even
// where |x| >> |dx|; W, the grad-W factor and every pair sum are FP32, the sums
// Kahan-compensated. The per-particle work that decides accuracy stays FP64:
// the EoS Newton inversion, pi^{mu nu} reconstruction, the RK2 state update
// and the conservation sums; the equations of motion run in FP32.
//
// FP64 on this part is a narrow pipe (one FP64 warp instruction costs as much
// pipe time as 64 FP32 ones), so moving the pair loops off it removes the
// bound the FP64 passes sit on. The neighbour set is decided by the FP32
// predicate; pairs it classifies differently from the FP64 predicate lie at
// |r_a - r_b| = 2h to FP32 rounding, where W and grad W vanish as (2 - q)^3
// and (2 - q)^2.
#include "kernels.cuh"
#include "passes.cuh"
#include "physics.cuh"

namespace ccake {

namespace {

using namespace passes;

// Packs the mixed smoothing record from the FP64 state (before the first
// mixed substep, and whenever FP64 passes moved the particles last).
template <int D>
__global__ void k_pack_mixed(Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const double x[3] = {p.y[Y_X0 * n + i], p.y[Y_X1 * n + i], D == 3 ? p.y[Y_X2 * n + i] : 0.0};
  const double ext[4] = {p.y[Y_ES * n + i], p.y[Y_EB * n + i], p.y[Y_ESS * n + i], p.y[Y_EQ * n + i]};
  write_recAf<D>(p, i, x, p.m[i], ext);
}

// Pass A, mixed form: smoothing sums (sigma_lab and the four extensive
// densities, src/sph_workstation.cpp:495-578 of the reference) over the
// candidate list, and the per-substep neighbour list with FP32 grad-W
// factors for pass B.
//
// The list is k-major (entry k of particle i at k * n + i) so that pass B
// reads it coalesced. The lanes of a warp reach entry k at different
// candidates; in 3-D (~450 entries a particle) the entries are staged in a
// per-warp ring of kRing rows in shared memory and each row is stored as one
// coalesced row once every lane still walking candidates has passed it
// (checked every kCheck candidates). A lane that would run more than kRing
// rows ahead of the slowest forces out the oldest rows; entries of a lane
// that is behind an already written row go straight to memory. In 2-D (~48
// entries) the entries are stored directly.
constexpr int kRing = 16, kCheck = 4;

template <int D>
__device__ __forceinline__ void passA_mixed_body(const RunConst& rc, const Ptrs& p, const int i_) {
  constexpr bool kStage = (D == 3);
  // every lane of a warp takes part in the warp-wide staging below: lanes
  // past the end stay in with no candidates and write nothing
  const int n = p.n;
  const bool live = i_ < n;
  const int i = live ? i_ : n - 1;
  const double t = p.clock->t;
  const float4* ra = reinterpret_cast<const float4*>(p.recAf);
  constexpr int SA = raf_stride<D>() / 4;
  const float4 ah = ra[(size_t)i * SA], al = ra[(size_t)i * SA + 1], ae = ra[(size_t)i * SA + 2];
  const float k0 = rc.fk0;
  KSum sl, s0, s1, s2, s3;
  sl.init(ah.w * k0);
  s0.init(ae.x * k0);
  s1.init(ae.y * k0);
  s2.init(ae.z * k0);
  s3.init(ae.w * k0);
  const float cut2 = rc.fcut2, ih = rc.finv_h;
  const float wn = rc.fwn, wn2 = rc.fwn2, gn = rc.fgn, gn2 = rc.fgn2;
  const int K = p.K;
  float* nf = reinterpret_cast<float*>(p.nbr_f);
  // a lane reads and writes only its own column of the ring (dynamically
  // indexed per-lane storage); the warp agrees on base by reductions
  __shared__ int ring_b[kBlock / 32][kRing][32];
  __shared__ float ring_f[kBlock / 32][kRing][32];
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  // stores row r of the ring for every lane that has an entry there
  int nn = 0, base = 0;
  int32_t* const nidx = p.nbr_idx;
  const int32_t* const cand = p.cand_idx;
  auto flush_row = [&](int r) {
    if (nn > r && r < K) {
      nidx[(size_t)r * n + i] = ring_b[wq][r % kRing][lane];
      nf[(size_t)r * n + i] = ring_f[wq][r % kRing][lane];
    }
  };
  // the candidate list of the last build holds every b that can be within
  // 2h now (most are); its entries are streamed two iterations ahead of use
  const int nc = live ? min(p.cand_cnt[i], p.Kc) : 0;
  const int wnc = kStage ? __reduce_max_sync(0xffffffffu, nc) : nc;
  int bq0 = 0, bq1 = 0;
  if (nc > 0) bq0 = cand[i];
  if (nc > 1) bq1 = cand[(size_t)n + i];
  for (int kk = 0; kk < wnc; kk++) {
    const bool act = kk < nc;
    if (kStage && (kk % kCheck) == 0) {
      // rows every lane still walking has passed are complete
      const int lo = __reduce_min_sync(0xffffffffu, act ? nn : 0x7fffffff);
      while (base < lo && lo != 0x7fffffff) {
        flush_row(base);
        base++;
      }
      // room for kCheck more rows a lane: the ring holds base .. base + kRing - 1
      const int hi = __reduce_max_sync(0xffffffffu, nn);
      while (hi + kCheck > base + kRing) {
        flush_row(base);
        base++;
      }
    }
    const int b = bq0;
    bq0 = bq1;
    if (kk + 2 < nc) bq1 = cand[(size_t)(kk + 2) * n + i];
    bool in = false;
    float fg = 0.0f;
    if (act) {
      float4 bh, bl;
      if (D == 3) {
        ldg256(&ra[(size_t)b * SA], bh, bl);
      } else {
        bh = __ldg(&ra[(size_t)b * SA]);
        bl = __ldg(&ra[(size_t)b * SA + 1]);
      }
      const float dx = (ah.x - bh.x) + (al.x - bl.x);
      const float dy = (ah.y - bh.y) + (al.y - bl.y);
      const float dz = (D == 3) ? (ah.z - bh.z) + (al.z - bl.z) : 0.0f;
      const float d2 = pair_d2f(dx, dy, dz);
      if (d2 <= cut2) {
        in = true;
        const float4 be = __ldg(&ra[(size_t)b * SA + 2]);
        // W (src/kernel.cpp:34-48) and grad_a W = fg (r_a - r_b) (:95-118)
        const float rs = d2 > 0.0f ? rsqrt_hw(d2) : 0.0f;
        const float q = d2 * rs * ih;
        const float z = fmaxf(2.0f - q, 0.0f), qq = q * q;
        const float W = q < 1.0f ? wn * (1.0f - 1.5f * qq + 0.75f * q * qq) : wn2 * z * z * z;
        fg = pair_fgf(d2, rs, ih, gn, gn2);
        sl.add(bh.w * W);
        s0.add(be.x * W);
        s1.add(be.y * W);
        s2.add(be.z * W);
        s3.add(be.w * W);
      }
    }
    if constexpr (kStage) {
      if (in) {
        if (nn < base) {
          if (nn < K) {
            nidx[(size_t)nn * n + i] = b;
            nf[(size_t)nn * n + i] = fg;
          }
        } else {
          ring_b[wq][nn % kRing][lane] = b;
          ring_f[wq][nn % kRing][lane] = fg;
        }
        nn++;
      }
    } else if (in) {
      if (nn < K) {
        nidx[(size_t)nn * n + i] = b;
        nf[(size_t)nn * n + i] = fg;
      }
      nn++;
    }
  }
  if constexpr (kStage) {
    const int hi = __reduce_max_sync(0xffffffffu, nn);
    while (base < hi) {
      flush_row(base);
      base++;
    }
  }
  if (!live) return;
  if (nn > K) flag_error(p.err, E_NBR_OVERFLOW);
  const double u3[3] = {p.y[Y_U0 * n + i], p.y[Y_U1 * n + i], D == 3 ? p.y[Y_U2 * n + i] : 0.0};
  const double tm = rc.cfg.coord == 1 ? 1.0 : t;   // the metric's tau (1 in Cartesian coordinates)
  const double g = gamma_milne<D>(u3, tm * tm);
  p.gam[i] = g;
  const double ig = 1.0 / g, igt = 1.0 / (g * tm);
#pragma unroll
  for (int q = 0; q < 3; q++) p.v[q * n + i] = (q < D) ? u3[q] * ig : 0.0;
  const double slab = sl.value64();
  p.slab[i] = slab;
  p.sig[i] = slab * igt;
  p.th[T_S * n + i] = s0.value64() * igt;
  p.th[T_RB * n + i] = s1.value64() * igt;
  p.th[T_RS * n + i] = s2.value64() * igt;
  p.th[T_RQ * n + i] = s3.value64() * igt;
  p.btrack[i] = nn;
}

// EoS inversion and the mixed gradient record, as a kernel of its own: the
// FP64 Newton solve needs ~255 registers a thread, which would cap the
// occupancy of the gather loop above at 8 warps an SM.
template <int D, bool DIFF>
__device__ __forceinline__ void thermo_mixed_body(const RunConst& rc, const EosDev& eos, const Ptrs& p, const int i,
                                                  bool pending_only) {
  if (i >= p.n) return;
  if (pending_only && p.eos_iters[i] != kEosPending) return;
  thermo_tail<D, true, DIFF>(rc, eos, p, i, p.clock->t);
}

// The EoS pass of the mixed form for the analytic models (conformal and
// conformal-diagonal, no pre-inverted tables): eos_invert's first attempt in
// seed mode 1 -- the exact inverse, accepted by the reference's residual
// test -- settles every particle it can, in a kernel a fraction of the full
// inverter's size (more warps an SM for the FP64 pipe to draw on). The
// particles it does not settle, and every particle of a table EoS, are
// marked pending for the full inversion (k_thermo_mixed with pending_only),
// which starts over from the same state: the results are eos_invert's.
template <int D, bool DIFF>
__device__ __forceinline__ void thermo_fast_body(const RunConst& rc, const EosDev& eos, const Ptrs& p, const int i) {
  if (i >= p.n) return;
  const int n = p.n;
  double x[4], o[17];
  int k = -2;
  if (!eos.pre) {
    const double tgt[4] = {p.th[T_S * n + i], p.th[T_RB * n + i], p.th[T_RS * n + i], p.th[T_RQ * n + i]};
    k = eos_analytic_first(eos, tgt, p.eos_id[i], x, o);
  }
  if (k < 0) {
    p.eos_iters[i] = kEosPending;
    return;
  }
  double th[NTH];
  set_thermo_o(eos, k, x, o, th, true);
  if constexpr (DIFF) {
    double da[12];
    alpha_derivs_o(eos, k, x, o, da);
#pragma unroll
    for (int q = 0; q < 12; q++) p.dif[(size_t)(F_DA + q) * n + i] = da[q];
  }
  thermo_store<D, true, DIFF>(rc, p, i, p.clock->t, th, k, 0);
}

// Diffusion sums of the mixed form, for particle i: the separable sums of
// k_diffgrad (src/sph_workstation.cpp:909-967 of the reference: v.grad q^0,
// div q and grad alpha of each charge) in FP32 with Kahan compensation over
// the FP32 list, from the FP32 records: positions as (hi, lo) pairs and the
// mass from record B, the diffusion record in the first half of its slot.
// The particle's own values come from the same records as its neighbours'.
// Written to the FP64 diffusion slabs the equations of motion read.
template <int D>
__device__ __forceinline__ void diffgrad_mixed_body(const Ptrs& p, const int i) {
  if (i >= p.n) return;
  const int n = p.n;
  constexpr int SB = RBF / 4;
  const float4* rbf = reinterpret_cast<const float4*>(p.recBf);
  const float4 A0 = rbf[(size_t)i * SB], A1 = rbf[(size_t)i * SB + 1], A2 = rbf[(size_t)i * SB + 2];
  const float va[3] = {A2.z, A2.w, D == 3 ? rbf[(size_t)i * SB + 3].x : 0.0f};
  // the diffusion record: two 32-byte loads (the slot is 128-byte aligned)
  auto rec = [&](int b, float* f) {
    const float4* rq = reinterpret_cast<const float4*>(p.recQ + (size_t)b * RQ);
    float4 v[4];
    ldg256(rq, v[0], v[1]);
    ldg256(rq + 2, v[2], v[3]);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) {
      f[4 * k2] = v[k2].x; f[4 * k2 + 1] = v[k2].y; f[4 * k2 + 2] = v[k2].z; f[4 * k2 + 3] = v[k2].w;
    }
  };
  KSum S1[D], SQ0[3][D], SA[3][D], SQI[3];
#pragma unroll
  for (int k = 0; k < D; k++) {
    S1[k].init(0.0f);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      SQ0[c][k].init(0.0f);
      SA[c][k].init(0.0f);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) SQI[c].init(0.0f);
  const float* nf = reinterpret_cast<const float*>(p.nbr_f);
  const int32_t* nidx = p.nbr_idx;
  const int cnt = min(p.btrack[i], p.K);
  // list entries streamed one iteration ahead of use
  int bq = cnt > 0 ? nidx[i] : 0;
  float fq = cnt > 0 ? nf[i] : 0.0f;
  for (int kk = 0; kk < cnt; kk++) {
    const int b = bq;
    const float fg = fq;
    if (kk + 1 < cnt) {
      bq = nidx[(size_t)(kk + 1) * n + i];
      fq = nf[(size_t)(kk + 1) * n + i];
    }
    float4 B0, B1;
    ldg256(rbf + (size_t)b * SB, B0, B1);
    const float d[3] = {(A0.x - B0.x) + (A1.x - B1.x), (A0.y - B0.y) + (A1.y - B1.y),
                        (D == 3) ? (A0.z - B0.z) + (A1.z - B1.z) : 0.0f};
    const float mf = B0.w * fg;
    float gm[D];
#pragma unroll
    for (int k = 0; k < D; k++) gm[k] = mf * d[k];
    float f[16];
    rec(b, f);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < D; k++) {
        SQ0[c][k].add(f[c] * gm[k]);
        SA[c][k].add(f[3 + c] * gm[k]);
        acc += f[6 + 3 * k + c] * gm[k];
      }
      SQI[c].add(acc);
    }
#pragma unroll
    for (int k = 0; k < D; k++) S1[k].add(gm[k]);
  }
  float fa[16];
  rec(i, fa);
  const float sla = f32_rn(p.slab[i]), isla = 1.0f / sla;
  float s1[D], vS1 = 0.0f;
#pragma unroll
  for (int k = 0; k < D; k++) {
    s1[k] = S1[k].value();
    vS1 += va[k] * s1[k];
  }
  double* df = p.dif;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    float vq = 0.0f, qs = 0.0f;
#pragma unroll
    for (int k = 0; k < D; k++) {
      vq += va[k] * SQ0[c][k].value();
      qs += fa[6 + 3 * k + c] * s1[k];
    }
    df[(size_t)(F_GQ + c) * n + i] = f64_of(sla * (vq + fa[c] * vS1));
    df[(size_t)(F_DQ + c) * n + i] = f64_of(sla * (SQI[c].value() + qs));
#pragma unroll
    for (int k = 0; k < 3; k++)
      df[(size_t)(F_GA + 3 * k + c) * n + i] = (k < D) ? f64_of((SA[c][k].value() - fa[3 + c] * s1[k]) * isla) : 0.0;
  }
}

// Pass B, mixed form, part 1: separable gradient sums over the list pass A
// wrote, FP32 with Kahan compensation (the separable forms of
// src/sph_workstation.cpp:797-986), written to the float view of the gradient
// slab (slot q of particle i at q * n + i, slots as GradSlot). The equations
// of motion run in k_eom_mixed: kept apart, this gather loop needs ~70
// registers a thread instead of ~170 and keeps enough warps in flight to
// cover its gather latency.
template <int D>
__device__ __forceinline__ void passB_mixed_body(const RunConst& rc, const Ptrs& p, const int i) {
  if (i >= p.n) return;
  const int n = p.n;
  const bool shear = rc.cfg.using_shear;
  constexpr int SB = RBF / 4;
  const float4* rbf = reinterpret_cast<const float4*>(p.recBf);
  const float4 A0 = rbf[(size_t)i * SB], A1 = rbf[(size_t)i * SB + 1], A2 = rbf[(size_t)i * SB + 2];
  const float4 A3 = rbf[(size_t)i * SB + 3], A4 = rbf[(size_t)i * SB + 4], A5 = rbf[(size_t)i * SB + 5];
  KSum S1[D], SP[D], SE[D], SB_[D], SV[D][D], S0[D][D], SD[D];
#pragma unroll
  for (int k = 0; k < D; k++) {
    S1[k].init(0.0f);
    SP[k].init(0.0f);
    SE[k].init(0.0f);
    SB_[k].init(0.0f);
    SD[k].init(0.0f);
#pragma unroll
    for (int l = 0; l < D; l++) {
      SV[k][l].init(0.0f);
      S0[k][l].init(0.0f);
    }
  }
  const float* nf = reinterpret_cast<const float*>(p.nbr_f);
  const int cnt = min(p.btrack[i], p.K);
  // the list entries are streamed from memory two iterations ahead of use
  int bq0 = 0, bq1 = 0;
  float fq0 = 0.0f, fq1 = 0.0f;
  // and, in 2-D, the first 32 bytes of the next neighbour's record one
  // ahead (in 3-D the extra registers would cost a block an SM)
  constexpr bool kAhead = (D == 2);
  float4 N0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), N1 = N0;
  if (cnt > 0) {
    bq0 = p.nbr_idx[i];
    fq0 = nf[i];
    if (kAhead) ldg256(rbf + (size_t)bq0 * SB, N0, N1);
  }
  if (cnt > 1) { bq1 = p.nbr_idx[(size_t)n + i]; fq1 = nf[(size_t)n + i]; }
  for (int kk = 0; kk < cnt; kk++) {
    const int b = bq0;
    const float fg = fq0;
    float4 B0 = N0, B1 = N1;
    if (kAhead) {
      if (kk + 1 < cnt) ldg256(rbf + (size_t)bq1 * SB, N0, N1);
    } else {
      ldg256(rbf + (size_t)b * SB, B0, B1);
    }
    bq0 = bq1;
    fq0 = fq1;
    if (kk + 2 < cnt) {
      bq1 = p.nbr_idx[(size_t)(kk + 2) * n + i];
      fq1 = nf[(size_t)(kk + 2) * n + i];
    }
    const float4* rb = rbf + (size_t)b * SB;
    float4 B2, B3 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (D == 3 || shear) ldg256(rb + 2, B2, B3);
    else B2 = __ldg(rb + 2);
    const float d[3] = {(A0.x - B0.x) + (A1.x - B1.x), (A0.y - B0.y) + (A1.y - B1.y),
                        (D == 3) ? (A0.z - B0.z) + (A1.z - B1.z) : 0.0f};
    const float mf = B0.w * fg;
    float gm[D];
#pragma unroll
    for (int k = 0; k < D; k++) gm[k] = mf * d[k];
    float vb[3] = {B2.z, B2.w, 0.0f};
    if (D == 3) vb[2] = B3.x;
#pragma unroll
    for (int k = 0; k < D; k++) {
      S1[k].add(gm[k]);
      SP[k].add(B1.w * gm[k]);
      SE[k].add(B2.x * gm[k]);
      SB_[k].add(B2.y * gm[k]);
#pragma unroll
      for (int l = 0; l < D; l++) SV[k][l].add(vb[l] * gm[k]);
    }
    if (shear) {
      float4 B4, B5 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (D == 3) ldg256(rb + 4, B4, B5);
      else B4 = __ldg(rb + 4);
      const float p0[3] = {B3.y, B3.z, B3.w};
      // pi^{ij}/sl^2 packed (11 12 13 22 23 33)
      const float pij[6] = {B4.x, B4.y, B4.z, B4.w, B5.x, B5.y};
#pragma unroll
      for (int k = 0; k < D; k++) {
#pragma unroll
        for (int l = 0; l < D; l++) S0[k][l].add(p0[l] * gm[k]);
        float acc = 0.0f;
#pragma unroll
        for (int l = 0; l < D; l++) {
          const int lo = k < l ? k : l, hi = k < l ? l : k;
          acc += pij[lo == 0 ? hi : (lo == 1 ? 2 + hi : 5)] * gm[l];
        }
        SD[k].add(acc);
      }
    }
  }
  // own values from the same FP32 record as the neighbours', so that a
  // uniform field gives a zero gradient up to the compensated sums' error
  const float sla = f32_rn(p.slab[i]), isla = 1.0f / sla;
  const float ea = A2.x, Pa = A1.w, Pia = A2.y;
  const float va[3] = {A2.z, A2.w, D == 3 ? A3.x : 0.0f};
  const float pi0a[3] = {A3.y, A3.z, A3.w};
  const float pija[6] = {A4.x, A4.y, A4.z, A4.w, A5.x, A5.y};
  float s1v[D];
#pragma unroll
  for (int k = 0; k < D; k++) s1v[k] = S1[k].value();
  float gP[3] = {0, 0, 0}, gE[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gS[3] = {0, 0, 0}, dS[3] = {0, 0, 0};
  float gV[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float vS1 = 0.0f;
#pragma unroll
  for (int k = 0; k < D; k++) vS1 += va[k] * s1v[k];
#pragma unroll
  for (int k = 0; k < D; k++) {
    gP[k] = sla * (SP[k].value() + Pa * s1v[k]);
    gE[k] = (SE[k].value() - ea * s1v[k]) * isla;
    gB[k] = sla * (SB_[k].value() + Pia * s1v[k]);
#pragma unroll
    for (int l = 0; l < D; l++) gV[k * D + l] = (SV[k][l].value() - va[l] * s1v[k]) * isla;
    if (shear) {
      float acc = 0.0f;
#pragma unroll
      for (int l = 0; l < D; l++) acc += va[l] * S0[l][k].value();
      gS[k] = sla * (acc + pi0a[k] * vS1);
      float acc2 = SD[k].value();
#pragma unroll
      for (int l = 0; l < D; l++) {
        const int lo = k < l ? k : l, hi = k < l ? l : k;
        acc2 += pija[lo == 0 ? hi : (lo == 1 ? 2 + hi : 5)] * s1v[l];
      }
      dS[k] = sla * acc2;
    }
  }
  float* gf = reinterpret_cast<float*>(p.grads);
#pragma unroll
  for (int k = 0; k < D; k++) {
    gf[(G_P + k) * n + i] = gP[k];
    gf[(G_E + k) * n + i] = gE[k];
    gf[(G_B + k) * n + i] = gB[k];
    gf[(G_SH + k) * n + i] = gS[k];
    gf[(G_DS + k) * n + i] = dS[k];
  }
#pragma unroll
  for (int k = 0; k < D * D; k++) gf[(G_V + k) * n + i] = gV[k];
}

// Pass B, mixed form, part 2: FP32 equations of motion from the gradients of
// part 1, FP64 RK2 update, mixed smoothing record for the next substep.
template <int D, bool DIFF>
__device__ __forceinline__ void eom_mixed_body(const RunConst& rc, const Ptrs& p, const int i, const int mode,
                                               const double dt_sub) {
  if (i >= p.n) return;
  const int n = p.n;
  const float* gf = reinterpret_cast<const float*>(p.grads);
  const float4 A2 = reinterpret_cast<const float4*>(p.recBf)[(size_t)i * (RBF / 4) + 2];
  const float va[3] = {A2.z, A2.w, D == 3 ? p.recBf[(size_t)i * RBF + 12] : 0.0f};
  float gP[3] = {0, 0, 0}, gE[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gS[3] = {0, 0, 0}, dS[3] = {0, 0, 0};
  float gV[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < D; k++) {
    gP[k] = gf[(G_P + k) * n + i];
    gE[k] = gf[(G_E + k) * n + i];
    gB[k] = gf[(G_B + k) * n + i];
    gS[k] = gf[(G_SH + k) * n + i];
    dS[k] = gf[(G_DS + k) * n + i];
  }
#pragma unroll
  for (int k = 0; k < D * D; k++) gV[k] = gf[(G_V + k) * n + i];
  finish_particle<D, float, true, DIFF>(rc, p, i, mode & ~B_GRADS, p.clock->t, dt_sub, va, gP, gE, gB, gS, dS, gV);
}

// ---------------------------------------------------------------------------
// grouped launches (GroupArgs): the events' descriptors in parameter space
// ---------------------------------------------------------------------------
// The event of this block (first_block is ascending; at most kGroupMax
// uniform comparisons), or -1 when that event is retired.
__device__ __forceinline__ int group_event(const GroupArgs& g, int& first) {
  int e = 0;
#pragma unroll 1
  while (e + 1 < g.nev && (int)blockIdx.x >= g.first_block[e + 1]) e++;
  first = ((int)blockIdx.x - g.first_block[e]) * kBlock;
  return g.state[e].active ? e : -1;
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_passA_mixed(const __grid_constant__ GroupArgs g) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  passA_mixed_body<D>(g.ev[e].rc, g.ev[e].p, first + threadIdx.x);
}

// The 3-D launch: declared for at least one block an SM, the candidate loop
// is scheduled with 64 registers instead of 46, which holds the SM at 8
// blocks instead of 10; the ring then takes 128 KB of shared memory instead
// of 160 KB and leaves the gathers a larger L1 (3-D pass A 12.6 -> 11.4 ms
// at 1.44M particles). The 2-D step runs 2 % slower with its loop so
// declared (60 registers), so it keeps the plain bound.
template <int D>
__global__ void __launch_bounds__(kBlock, 1) k_passA_mixed_wide(const __grid_constant__ GroupArgs g) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  passA_mixed_body<D>(g.ev[e].rc, g.ev[e].p, first + threadIdx.x);
}

template <int D, bool DIFF>
__global__ void __launch_bounds__(kBlock) k_thermo_fast(const __grid_constant__ GroupArgs g) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  thermo_fast_body<D, DIFF>(g.ev[e].rc, g.ev[e].eos, g.ev[e].p, first + threadIdx.x);
}

template <int D, bool DIFF>
__global__ void __launch_bounds__(kBlock) k_thermo_mixed(const __grid_constant__ GroupArgs g, int pending_only) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  thermo_mixed_body<D, DIFF>(g.ev[e].rc, g.ev[e].eos, g.ev[e].p, first + threadIdx.x, pending_only != 0);
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_diffgrad_mixed(const __grid_constant__ GroupArgs g) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  diffgrad_mixed_body<D>(g.ev[e].p, first + threadIdx.x);
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_passB_mixed(const __grid_constant__ GroupArgs g) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  passB_mixed_body<D>(g.ev[e].rc, g.ev[e].p, first + threadIdx.x);
}

// The 3-D launch: its gather loop holds ~140 registers a thread, 3 blocks an
// SM; held to 128 it keeps 4 blocks (16 warps) in flight for the L1-bound
// gathers (3-D pass B 7.6 -> 6.5 ms at 1.44M particles). The 2-D loop runs
// slower under the same bound, so it keeps the plain one.
template <int D>
__global__ void __launch_bounds__(kBlock, 4) k_passB_mixed_r128(const __grid_constant__ GroupArgs g) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  passB_mixed_body<D>(g.ev[e].rc, g.ev[e].p, first + threadIdx.x);
}

template <int D, bool DIFF>
__global__ void __launch_bounds__(kBlock) k_eom_mixed(const __grid_constant__ GroupArgs g, int mode, int sub) {
  int first;
  const int e = group_event(g, first);
  if (e < 0) return;
  const double dt = g.ev[e].rc.cfg.dt;
  eom_mixed_body<D, DIFF>(g.ev[e].rc, g.ev[e].p, first + threadIdx.x, mode, sub == 1 ? 0.5 * dt : dt);
}

__global__ void k_clock_group(const __grid_constant__ GroupArgs g, int sub) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.nev || !g.state[k].active) return;
  advance_clock(g.ev[k].p.clock, sub, g.ev[k].rc.cfg.dt);
  if (sub == 2) g.state[k].steps++;
}

__global__ void __launch_bounds__(kBlock) k_freeze_group(const __grid_constant__ GroupArgs g) {
  int first;
  const int e = group_event(g, first);
  if (e < 0 || !g.ev[e].rc.cfg.particlization) return;
  freeze_particle(g.ev[e].rc, g.ev[e].p, first + threadIdx.x);
}

__global__ void k_freeze_advance_group(const __grid_constant__ GroupArgs g) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.nev || !g.state[k].active || !g.ev[k].rc.cfg.particlization) return;
  Clock* c = g.ev[k].p.clock;
  if (c->frzc < 2) c->frzc++;
}

// The stop rule before a step, one block an event: SPHWorkstation::
// continue_evolution (src/sph_workstation.cpp:1992-2024: every particle frozen
// out with particlization), the event's tau_max, and the failures the kernels
// flagged (the first one decides the status). Idempotent: it may run again
// with no step in between.
__global__ void __launch_bounds__(256) k_stop_group(const __grid_constant__ GroupArgs g) {
  EventState& E = g.state[blockIdx.x];
  if (!E.active) return;
  const Ptrs& p = g.ev[blockIdx.x].p;
  const ccake_config& cfg = g.ev[blockIdx.x].rc.cfg;
  __shared__ int red[8];
  int frozen = 0;
  if (cfg.particlization)
    for (int i = threadIdx.x; i < p.n; i += blockDim.x) frozen += p.freeze[i] >= 4 ? 1 : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) frozen += __shfl_xor_sync(0xffffffffu, frozen, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = frozen;
  __syncthreads();
  if (threadIdx.x != 0) return;
  frozen = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) frozen += red[w];
  E.tau = p.clock->t;
  const int first = p.err[E_FIRST] - 1;
  const int kind[4] = {CCAKE_ERR_EOS, CCAKE_ERR_NEG_ENTROPY, CCAKE_ERR_NONFINITE, CCAKE_ERR_CAPACITY};
  if (first >= 0 && first < 4) {
    E.status = kind[first];
    E.active = 0;
  } else if (cfg.particlization && frozen >= p.n) {
    E.frozen_stop = 1;
    E.active = 0;
  } else if (p.clock->t >= E.tau_max - 0.5 * cfg.dt) {
    E.active = 0;
  }
}

}  // namespace

void launch_pack_mixed(const RunConst& rc, const Ptrs& p, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  if (rc.cfg.dim == 3) k_pack_mixed<3><<<nb, kBlock, 0, s>>>(p);
  else k_pack_mixed<2><<<nb, kBlock, 0, s>>>(p);
}

// The analytic EoS pass runs when an event of the group has an analytic
// model first in its chain (conformal, conformal-diagonal; no pre-inverted
// tables); the full inversion then takes only the particles it left.
static bool group_has_analytic(const GroupArgs& g) {
  for (int e = 0; e < g.nev; e++) {
    const EosDev& q = g.ev[e].eos;
    if (!q.pre && q.kind != 2) return true;
  }
  return false;
}

// A group with the diffusion sector (the server groups none; an event with
// it runs alone): every member has it on.
static bool group_has_diffusion(const GroupArgs& g) {
  for (int e = 0; e < g.nev; e++)
    if (g.ev[e].rc.cfg.using_diffusion && g.ev[e].p.dif) return true;
  return false;
}

void launch_passA_mixed(const GroupArgs& g, int dim, cudaStream_t s) {
  const int nb = g.first_block[g.nev];
  const bool dif = group_has_diffusion(g);
  const int fast = group_has_analytic(g) ? 1 : 0;
  if (dim == 3) {
    k_passA_mixed_wide<3><<<nb, kBlock, 0, s>>>(g);
    if (dif) {
      if (fast) k_thermo_fast<3, true><<<nb, kBlock, 0, s>>>(g);
      k_thermo_mixed<3, true><<<nb, kBlock, 0, s>>>(g, fast);
    } else {
      if (fast) k_thermo_fast<3, false><<<nb, kBlock, 0, s>>>(g);
      k_thermo_mixed<3, false><<<nb, kBlock, 0, s>>>(g, fast);
    }
  } else {
    k_passA_mixed<2><<<nb, kBlock, 0, s>>>(g);
    if (dif) {
      if (fast) k_thermo_fast<2, true><<<nb, kBlock, 0, s>>>(g);
      k_thermo_mixed<2, true><<<nb, kBlock, 0, s>>>(g, fast);
    } else {
      if (fast) k_thermo_fast<2, false><<<nb, kBlock, 0, s>>>(g);
      k_thermo_mixed<2, false><<<nb, kBlock, 0, s>>>(g, fast);
    }
  }
}

// With the diffusion sector its sums run first (they read the diffusion
// records of the neighbours, complete after the EoS kernel).
void launch_passB_mixed(const GroupArgs& g, int dim, int mode, int sub, cudaStream_t s) {
  const int nb = g.first_block[g.nev];
  const bool dif = group_has_diffusion(g);
  if (dim == 3) {
    if (dif) k_diffgrad_mixed<3><<<nb, kBlock, 0, s>>>(g);
    k_passB_mixed_r128<3><<<nb, kBlock, 0, s>>>(g);
    if (dif) k_eom_mixed<3, true><<<nb, kBlock, 0, s>>>(g, mode, sub);
    else k_eom_mixed<3, false><<<nb, kBlock, 0, s>>>(g, mode, sub);
  } else {
    if (dif) k_diffgrad_mixed<2><<<nb, kBlock, 0, s>>>(g);
    k_passB_mixed<2><<<nb, kBlock, 0, s>>>(g);
    if (dif) k_eom_mixed<2, true><<<nb, kBlock, 0, s>>>(g, mode, sub);
    else k_eom_mixed<2, false><<<nb, kBlock, 0, s>>>(g, mode, sub);
  }
}

void launch_gradients_mixed(const GroupArgs& g, int dim, cudaStream_t s) {
  const int nb = g.first_block[g.nev];
  if (dim == 3) k_passB_mixed_r128<3><<<nb, kBlock, 0, s>>>(g);
  else k_passB_mixed<2><<<nb, kBlock, 0, s>>>(g);
}

void launch_clock_group(const GroupArgs& g, int sub, cudaStream_t s) {
  k_clock_group<<<(g.nev + 127) / 128, 128, 0, s>>>(g, sub);
}

void launch_freeze_group(const GroupArgs& g, cudaStream_t s) {
  k_freeze_group<<<g.first_block[g.nev], kBlock, 0, s>>>(g);
  k_freeze_advance_group<<<(g.nev + 127) / 128, 128, 0, s>>>(g);
}

void launch_stop_group(const GroupArgs& g, cudaStream_t s) { k_stop_group<<<g.nev, 256, 0, s>>>(g); }

}  // namespace ccake
