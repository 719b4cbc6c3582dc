// Device pieces shared by the FP64 and the mixed-precision passes.
#pragma once
#include "kernels.cuh"
#include "physics.cuh"

namespace ccake {
namespace passes {

constexpr int kSurv = 64;   // candidate chunk kept per thread in shared memory (pass A)

// Row ranges [lo, hi) of the sorted cell list covering the 3^D neighbour
// cells of a position (the cells of one (y, z) row are contiguous).
template <int D>
__device__ __forceinline__ int neighbour_ranges(const Grid& gr, const int32_t* cell_start, const double* xa,
                                                int* rlo, int* rhi) {
  int nr = 0;
  const int cx = cell_coord(gr, 0, xa[0]), cy = cell_coord(gr, 1, xa[1]);
  const int cz = (D == 3) ? cell_coord(gr, 2, xa[2]) : 0;
  const int zlo = (D == 3) ? max(cz - 1, 0) : 0, zhi = (D == 3) ? min(cz + 1, gr.nc[2] - 1) : 0;
  for (int z = zlo; z <= zhi; z++)
    for (int y = max(cy - 1, 0); y <= min(cy + 1, gr.nc[1] - 1); y++) {
      const int row = (z * gr.nc[1] + y) * gr.nc[0];
      rlo[nr] = cell_start[row + max(cx - 1, 0)];
      rhi[nr] = cell_start[row + min(cx + 1, gr.nc[0] - 1) + 1];
      nr++;
    }
  return nr;
}

// FP32 screen of a candidate pair: false only when the FP32 squared distance
// exceeds (2h)^2 by more than a bound on its FP32 error (per axis
// 2^-22 (|x_a| + |x_b| + |dx|) before squaring, 4e-7 relative after), so every
// pair the exact FP64 predicate accepts survives. d2f returns the FP32
// squared distance, bound its error bound.
template <int D>
__device__ __forceinline__ bool maybe_neighbour(const float4& pa, const float4& pb, float cut2f, float& d2f,
                                                float& bound) {
  const float dxf = pa.x - pb.x, dyf = pa.y - pb.y, dzf = (D == 3) ? pa.z - pb.z : 0.0f;
  const float ex = 2.4e-7f * (fabsf(pa.x) + fabsf(pb.x) + fabsf(dxf)) + 1e-30f;
  const float ey = 2.4e-7f * (fabsf(pa.y) + fabsf(pb.y) + fabsf(dyf)) + 1e-30f;
  const float ez = (D == 3) ? 2.4e-7f * (fabsf(pa.z) + fabsf(pb.z) + fabsf(dzf)) + 1e-30f : 0.0f;
  d2f = dxf * dxf + dyf * dyf + dzf * dzf;
  bound = ex * (2.0f * fabsf(dxf) + ex) + ey * (2.0f * fabsf(dyf) + ey) + ez * (2.0f * fabsf(dzf) + ez) + 4e-7f * d2f;
  return !(d2f - bound > cut2f);
}

// Compensated (Kahan) FP32 sum: s - c carries the sum to about FP32
// precision of the sum itself rather than of the sum of magnitudes.
struct KSum {
  float s, c;
  __device__ __forceinline__ void init(float x) { s = x; c = 0.0f; }
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ float value() const { return s - c; }
  __device__ __forceinline__ double value64() const { return f64_of(s) - f64_of(c); }
};

// 1/sqrt(x) for normal x > 0 by the hardware approximation
// (rsqrt.approx.ftz.f32, about 2^-22.9 relative error): one special-function
// instruction. Pair distances squared are never subnormal (and zero is
// excluded by the callers).
__device__ __forceinline__ float rsqrt_hw(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// FP64 kernel values of one pair at squared distance d2 (>= 0, finite, at
// most cut2): W(r) (src/kernel.cpp:34-48 of the reference) and the radial
// factor fg of grad_a W = fg (r_a - r_b) (:95-118), fg = gn (2 - q)^2 / r for
// 1 <= q < 2 and gn2 (1.5 q - 2) / h for q < 1, q = r / h. The FP64 pipe
// bounds the FP64 passes, so this spends as few FP64 instructions as it can
// (17 a pair):
//  * 1/r: the FP32 hardware estimate y0 (rsqrt_hw, relative error d <=
//    2^-22.9 + 2^-24 for the truncated input) refined by the third-order
//    step of the binomial series y = y0 (1 - e)^(-1/2) = y0 (1 + e/2 +
//    3 e^2/8 + ...), e = 1 - d2 y0^2 (Householder's method of order 2 for
//    x^(-1/2)): the truncation error is about 5 |e|^3 / 16 = 2.5 d^3 < 1e-19,
//    so y is 1/r to within the few roundings of the step (~2 ulp).
//  * the FP64 <-> FP32 moves of the estimate are done on the IEEE bit
//    patterns by integer instructions (a hardware conversion is an FP64-pipe
//    instruction): d2 truncated to FP32, inputs below the smallest normal
//    FP32 number lifted to it (a zero distance still gives q = 0, W = wn);
//    the normal FP32 estimate widened exactly.
//  * both polynomial branches are evaluated and selected; q >= 0, so the
//    branch tests compare the high word of q on the integer pipe.
//  * every product and difference is rounded on its own (_rn intrinsics,
//    never contracted), so each branch's value does not depend on how the
//    caller reaches it (pair_kernel_warp below).
// The result is symmetric in the pair (it depends on d2 alone), so the pair
// sums keep the antisymmetry the conservation laws rest on.
// K: RunConst (the run's kernel) or KernelConst (a factor of the factorised
// 3-D kernel); the same member names.
template <class K>
__device__ __forceinline__ void pair_q(const K& rc, double d2, double& y, double& q) {
  const int hi = max(__double2hiint(d2), 897 << 20);
  const unsigned xf = __funnelshift_l((unsigned)__double2loint(d2), (unsigned)(hi - (896 << 20)), 3);
  const unsigned yb = __float_as_uint(rsqrt_hw(__uint_as_float(xf)));
  const double y0 = __hiloint2double((int)((yb >> 3) + (896u << 20)), (int)(yb << 29));
  const double e = fma(-__dmul_rn(d2, y0), y0, 1.0);
  y = fma(y0, __dmul_rn(e, fma(0.375, e, 0.5)), y0);   // 1/r
  q = __dmul_rn(__dmul_rn(d2, y), rc.inv_h);
}

// q < 1 (src/kernel.cpp:40-44, :103-106)
template <class K>
__device__ __forceinline__ void pair_inner(const K& rc, double q, double& W, double& fg) {
  W = fma(__dmul_rn(q, q), fma(rc.win_c2, q, rc.win_c1), rc.wn);
  fg = fma(rc.fin_a, q, rc.fin_b);
}

// 1 <= q < 2 (src/kernel.cpp:45-47, :107-112)
template <class K>
__device__ __forceinline__ void pair_outer(const K& rc, double q, double y, double& W, double& fg) {
  const double z = __dsub_rn(2.0, q), z2 = __dmul_rn(z, z);
  W = __dmul_rn(__dmul_rn(rc.wn2, z), z2);
  fg = __dmul_rn(__dmul_rn(rc.gn, y), z2);
}

template <class K>
__device__ __forceinline__ void pair_kernel(const K& rc, double d2, double& W, double& fg) {
  double y, q, Win, fin, Wout, fout;
  pair_q(rc, d2, y, q);
  pair_inner(rc, q, Win, fin);
  pair_outer(rc, q, y, Wout, fout);
  const int qh = __double2hiint(q);
  const bool in1 = qh < 0x3FF00000, in2 = qh < 0x40000000;   // q < 1, q < 2
  W = in1 ? Win : (in2 ? Wout : 0.0);
  fg = in1 ? fin : (in2 ? fout : 0.0);
}

// pair_kernel for a warp: when every active lane is on the same side of
// q = 1, only that side's polynomial runs (6 or 4 FP64 instructions fewer a
// pair; the candidate lists put the pairs within h first, so on a lattice
// the lanes of a warp mostly agree). The same operations as pair_kernel on
// each side, hence the same bits whichever path a lane takes.
template <class K>
__device__ __forceinline__ void pair_kernel_warp(const K& rc, double d2, double& W, double& fg) {
  double y, q;
  pair_q(rc, d2, y, q);
  const int qh = __double2hiint(q);
  const bool in1 = qh < 0x3FF00000, in2 = qh < 0x40000000;   // q < 1, q < 2
  const unsigned act = __activemask();
  if (__all_sync(act, in1)) {
    pair_inner(rc, q, W, fg);
  } else if (__all_sync(act, !in1)) {
    double Wo, fo;
    pair_outer(rc, q, y, Wo, fo);
    W = in2 ? Wo : 0.0;
    fg = in2 ? fo : 0.0;
  } else {
    double Win, fin, Wout, fout;
    pair_inner(rc, q, Win, fin);
    pair_outer(rc, q, y, Wout, fout);
    W = in1 ? Win : (in2 ? Wout : 0.0);
    fg = in1 ? fin : (in2 ? fout : 0.0);
  }
}

// Squared FP32 pair distance and the radial factor fg of grad_a W =
// fg (r_a - r_b) (src/kernel.cpp:95-118 of the reference), every rounding
// explicit (no contraction), so that the mixed pass A's predicate and pass
// B's recomputation from the same float positions agree bit for bit.
__device__ __forceinline__ float pair_d2f(float dx, float dy, float dz) {
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

__device__ __forceinline__ float pair_fgf(float d2, float rs, float ih, float gn, float gn2) {
  const float q = __fmul_rn(__fmul_rn(d2, rs), ih);
  const float z = fmaxf(__fsub_rn(2.0f, q), 0.0f);
  return q < 1.0f ? __fmul_rn(__fmul_rn(gn2, __fmaf_rn(1.5f, q, -2.0f)), ih)
                  : __fmul_rn(__fmul_rn(__fmul_rn(gn, rs), z), z);
}

// 32-byte load through the non-coherent path (ld.global.nc.v8.f32, sm_100
// and later): one gather instruction for two float4 of a neighbour record.
// p must be 32-byte aligned.
__device__ __forceinline__ void ldg256(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

// x = hi + lo with hi = fl32(x): the pair carries x to ~2^-48 relative.
__device__ __forceinline__ void split2(double x, float& hi, float& lo) {
  hi = f32_rn(x);
  lo = f32_rn(x - f64_of(hi));
}

// Smoothing record of particle i (FP64 form, plus the FP32 screen copy).
template <int D>
__device__ __forceinline__ void write_recA(const Ptrs& p, int i, const double* x, double m, const double* ext) {
  double2* ra = reinterpret_cast<double2*>(p.recA) + (size_t)i * 4;
  ra[0] = make_double2(x[0], x[1]);
  ra[1] = make_double2(D == 3 ? x[2] : 0.0, m);
  ra[2] = make_double2(m * ext[0], m * ext[1]);
  ra[3] = make_double2(m * ext[2], m * ext[3]);
  p.posf[i] = make_float4(f32_rn(x[0]), f32_rn(x[1]), D == 3 ? f32_rn(x[2]) : 0.0f, 0.0f);
}

// Smoothing record of particle i (mixed form).
template <int D>
__device__ __forceinline__ void write_recAf(const Ptrs& p, int i, const double* x, double m, const double* ext) {
  float hi[3], lo[3];
#pragma unroll
  for (int k = 0; k < 3; k++) split2(k < D ? x[k] : 0.0, hi[k], lo[k]);
  float4* ra = reinterpret_cast<float4*>(p.recAf) + (size_t)i * (raf_stride<D>() / 4);
  ra[0] = make_float4(hi[0], hi[1], hi[2], f32_rn(m));
  ra[1] = make_float4(lo[0], lo[1], lo[2], 0.0f);
  ra[2] = make_float4(f32_rn(m * ext[0]), f32_rn(m * ext[1]), f32_rn(m * ext[2]), f32_rn(m * ext[3]));
  if (D == 3) ra[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  p.posf[i] = make_float4(hi[0], hi[1], hi[2], 0.0f);
}

// EoS inversion of the smoothed densities of particle i, pi^{mu nu} and Pi
// from the extensive forms, and its gradient record (FP64 or mixed form).
// DIFF: the diffusion sector (FP64 form): the alpha derivatives at the
// solution, q^mu from the extensive current (src/eom_default.cpp:140-165),
// the regulator (src/sph_workstation.cpp:132-218) and the diffusion record.
template <int D, bool MIX, bool DIFF>
__device__ __forceinline__ void thermo_store(const RunConst& rc, const Ptrs& p, int i, double t, const double* th,
                                             int k, int iters);

template <int D, bool MIX, bool DIFF = false>
__device__ __forceinline__ void thermo_tail(const RunConst& rc, const EosDev& eos, const Ptrs& p, int i, double t) {
  const int n = p.n;
  double th[NTH];
  double x[4] = {p.th[T_T * n + i], p.th[T_MUB * n + i], p.th[T_MUQ * n + i], p.th[T_MUS * n + i]};
  const double tgt[4] = {p.th[T_S * n + i], p.th[T_RB * n + i], p.th[T_RS * n + i], p.th[T_RQ * n + i]};
  int iters = 0, k = 0;
  if (eos.pre) {
    // pre-inverted tables (EoS_Interpolator::fill_thermodynamics): the
    // densities stay, everything else is interpolated
    double v[kPreVars];
    preinv_lookup(*eos.pre, tgt, v);
    th[T_T] = v[PV_T];
    th[T_MUB] = v[PV_MUB];
    th[T_MUS] = v[PV_MUS];
    th[T_MUQ] = v[PV_MUQ];
    th[T_P] = v[PV_P];
    th[T_S] = tgt[0];
    th[T_RB] = tgt[1];
    th[T_RS] = tgt[2];
    th[T_RQ] = tgt[3];
    th[T_E] = v[PV_E];
    th[T_W] = v[PV_E] + v[PV_P];
    th[T_CS2] = v[PV_CS2];
    th[T_DWDS] = v[PV_DWDS];
    th[T_DWDB] = v[PV_DWDB];
    th[T_DWDSS] = v[PV_DWDS_S];
    th[T_DWDQ] = v[PV_DWDQ];
  } else {
    double o[17];
    k = eos_invert(eos, 1, tgt, p.eos_id[i], x, &iters, MIX ? 1 : 0, o);
    if (k < 0) {   // per-particle status: no EoS solution (the next search starts the chain over)
      p.eos_id[i] = -1;
      flag_error(p.err, E_EOS);
      return;
    }
    set_thermo_o(eos, k, x, o, th, MIX);
    if constexpr (DIFF) {
      double da[12];
      alpha_derivs_o(eos, k, x, o, da);
#pragma unroll
      for (int q = 0; q < 12; q++) p.dif[(size_t)(F_DA + q) * n + i] = da[q];
    }
  }
  thermo_store<D, MIX, DIFF>(rc, p, i, t, th, k, iters);
}

// Everything of the EoS pass after the inversion, for particle i with the
// thermodynamics th (chain index k, iters Newton steps): the stored
// thermodynamics, pi^{mu nu} and Pi from the extensive forms, and the
// gradient record (FP64 or mixed form; DIFF: the diffusion record).
template <int D, bool MIX, bool DIFF>
__device__ __forceinline__ void thermo_store(const RunConst& rc, const Ptrs& p, int i, double t, const double* th,
                                             int k, int iters) {
  const int n = p.n;
  const double t2 = rc.cfg.coord == 1 ? 1.0 : t * t;   // the metric's tau^2 (1 in Cartesian coordinates)
#pragma unroll
  for (int q = 0; q < NTH; q++) p.th[q * n + i] = th[q];
  p.eos_id[i] = k;
  p.eos_iters[i] = iters;
  // pi^{mu nu} and Pi from the extensive forms
  const double sig = p.sig[i], g = p.gam[i], slab = p.slab[i];
  double u3[3] = {p.y[Y_U0 * n + i], p.y[Y_U1 * n + i], D == 3 ? p.y[Y_U2 * n + i] : 0.0};
  double es[5];
#pragma unroll
  for (int q = 0; q < 5; q++) es[q] = p.y[(Y_SHV0 + q) * n + i];
  double pi[NPI];
  reset_pi<D>(es, sig, g, u3, t2, rc.cfg.coord == 1 ? 1.0 : p.clock->it2, pi);
  const double Pi = p.y[Y_EBULK * n + i] * sig;
  p.bulk[i] = Pi;
#pragma unroll
  for (int q = 0; q < NPI; q++) p.pi[q * n + i] = pi[q];
  // neighbour record B
  const double isl2 = 1.0 / (slab * slab);
  if constexpr (DIFF) {
    // q^i = ext q sigma, q^0 = -q^i u_i / gamma (u_i of the three-vector u
    // padded with zeros); then the regulator caps |q| at rq_max |n| f(e)
    const double fc[3] = {-u3[0], -u3[1], -t2 * u3[2]};
    double q[12];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double q0 = 0.;
#pragma unroll
      for (int k2 = 0; k2 < 3; k2++) q[4 * c + k2 + 1] = p.dif[(size_t)(F_YQ + 3 * c + k2) * n + i] * sig;
#pragma unroll
      for (int k2 = 0; k2 < 3; k2++) q0 += -q[4 * c + k2 + 1] * fc[k2] / g;
      q[4 * c] = q0;
    }
    if (rc.cfg.diffusion_regulator) {
      const double e0 = rc.cfg.reg_e0 / kHbarcGeVfm, xi0 = rc.cfg.reg_xi0 / kHbarcGeVfm;
      const double fermi_offset = 1.0 / (exp(e0 / xi0) + 1.0);
      const double ferm = 1.0 / (exp(-(th[T_E] - e0) / xi0) + 1.0);
      const double f_str = rc.cfg.reg_chi0 * (ferm - fermi_offset);
      const double rho[3] = {th[T_RB], th[T_RS], th[T_RQ]};
      for (int c = 0; c < 3; c++) {
        const double n_abs = fabs(rho[c]);
        if (n_abs < 1.0e-15) continue;
        const double q3_sq = rc.cfg.coord == 0 ? t2 * q[4 * c + 3] * q[4 * c + 3] : q[4 * c + 3] * q[4 * c + 3];
        const double q_sq = q[4 * c + 1] * q[4 * c + 1] + q[4 * c + 2] * q[4 * c + 2] + q3_sq - q[4 * c] * q[4 * c];
        if (q_sq <= 0.0) continue;
        const double q_mag = sqrt(q_sq);
        const double threshold = rc.cfg.reg_rq_max * n_abs * f_str;
        if (q_mag <= threshold) continue;
        const double scale = threshold / q_mag;
        for (int m = 0; m < 4; m++) q[4 * c + m] = q[4 * c + m] * scale;
      }
    }
    // the diffusion record of the neighbour sums: q^0/sl^2 (3), alpha = mu/T
    // (3), q^k/sl^2 (9); FP64, or FP32 in the first half of the same slot
    // (mixed form)
    double rv[16];
    const double iT = 1.0 / th[T_T];
#pragma unroll
    for (int c = 0; c < 3; c++) {
#pragma unroll
      for (int m = 0; m < 4; m++) p.dif[(size_t)(F_Q + 4 * c + m) * n + i] = q[4 * c + m];
      rv[c] = q[4 * c] * isl2;
#pragma unroll
      for (int k2 = 0; k2 < 3; k2++) rv[6 + 3 * k2 + c] = q[4 * c + k2 + 1] * isl2;
    }
    rv[3] = th[T_MUB] * iT;
    rv[4] = th[T_MUS] * iT;
    rv[5] = th[T_MUQ] * iT;
    rv[15] = 0.0;
    if constexpr (MIX) {
      float4* rq = reinterpret_cast<float4*>(p.recQ + (size_t)i * RQ);
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++)
        rq[k2] = make_float4(f32_rn(rv[4 * k2]), f32_rn(rv[4 * k2 + 1]), f32_rn(rv[4 * k2 + 2]), f32_rn(rv[4 * k2 + 3]));
    } else {
      double* rq = p.recQ + (size_t)i * RQ;
#pragma unroll
      for (int k2 = 0; k2 < 16; k2++) rq[k2] = rv[k2];
    }
  }
  if constexpr (MIX) {
    float hi[3], lo[3];
#pragma unroll
    for (int k = 0; k < 3; k++) split2(k < D ? p.y[(Y_X0 + k) * n + i] : 0.0, hi[k], lo[k]);
    const float f = f32_rn(isl2);
    float4* rb = reinterpret_cast<float4*>(p.recBf) + (size_t)i * (RBF / 4);
    rb[0] = make_float4(hi[0], hi[1], hi[2], f32_rn(p.m[i]));
    rb[1] = make_float4(lo[0], lo[1], lo[2], f32_rn(th[T_P] * isl2));
    rb[2] = make_float4(f32_rn(th[T_E]), f32_rn(Pi * isl2), f32_rn(p.v[i]), f32_rn(p.v[n + i]));
    rb[3] = make_float4(f32_rn(p.v[2 * n + i]), f32_rn(pi[pi_slot(0, 1)]) * f, f32_rn(pi[pi_slot(0, 2)]) * f,
                        f32_rn(pi[pi_slot(0, 3)]) * f);
    rb[4] = make_float4(f32_rn(pi[P11]) * f, f32_rn(pi[P12]) * f, f32_rn(pi[P13]) * f, f32_rn(pi[P22]) * f);
    rb[5] = make_float4(f32_rn(pi[P23]) * f, f32_rn(pi[P33]) * f, 0.0f, 0.0f);
  } else {
    double* rb = p.recB + (size_t)i * RB;
    rb[B_X0] = p.y[Y_X0 * n + i];
    rb[B_X1] = p.y[Y_X1 * n + i];
    rb[B_X2] = D == 3 ? p.y[Y_X2 * n + i] : 0.0;
    rb[B_M] = p.m[i];
    rb[B_P] = th[T_P] * isl2;
    rb[B_E] = th[T_E];
    rb[B_PI] = Pi * isl2;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      rb[B_V0 + q] = p.v[q * n + i];
      rb[B_PI0 + q] = pi[pi_slot(0, q + 1)] * isl2;
    }
    rb[B_PIJ + 0] = pi[P11] * isl2;
    rb[B_PIJ + 1] = pi[P12] * isl2;
    rb[B_PIJ + 2] = pi[P13] * isl2;
    rb[B_PIJ + 3] = pi[P22] * isl2;
    rb[B_PIJ + 4] = pi[P23] * isl2;
    rb[B_PIJ + 5] = pi[P33] * isl2;
  }
}

// Diffusion inputs of the equations of motion of particle i: q^mu, the
// alpha derivatives and the diffusion sums of the last evaluation, tau_q and
// kappa_q from its thermodynamics th.
__device__ __forceinline__ void load_diff_in(const RunConst& rc, const Ptrs& p, int i, const double* th,
                                             DiffIn& din) {
  const int n = p.n;
  const double* df = p.dif;
#pragma unroll
  for (int q = 0; q < 12; q++) {
    din.q[q] = df[(size_t)(F_Q + q) * n + i];
    din.da[q] = df[(size_t)(F_DA + q) * n + i];
  }
#pragma unroll
  for (int q = 0; q < 9; q++) din.ga[q] = df[(size_t)(F_GA + q) * n + i];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    din.gq[c] = df[(size_t)(F_GQ + c) * n + i];
    din.dq[c] = df[(size_t)(F_DQ + c) * n + i];
  }
  diffusion_coefs(rc.cfg, th, rc.cfg.eos_kind == 2 && p.eos_id[i] == 0, din.tq, din.kq);
}

// Everything of pass B after the gradients, for particle i: optional export
// of the gradients, the equations of motion (in type R), optional export of
// the derivatives, the midpoint RK2 update of the FP64 state from the
// step-start cache (reference src/evolver.cpp:344-486) and the smoothing
// record for the next substep (FP64 or mixed form).
template <int D, typename R, bool MIX, bool DIFF = false>
__device__ __forceinline__ void finish_particle(const RunConst& rc, const Ptrs& p, int i, int mode, double t,
                                                double dt_sub, const R* va, const R* gP, const R* gE, const R* gB,
                                                const R* gS, const R* dS, const R* gV) {
  const int n = p.n;
  if (mode & B_GRADS) {
#pragma unroll
    for (int k = 0; k < D; k++) {
      p.grads[(G_P + k) * n + i] = gP[k];
      p.grads[(G_E + k) * n + i] = gE[k];
      p.grads[(G_B + k) * n + i] = gB[k];
      p.grads[(G_SH + k) * n + i] = gS[k];
      p.grads[(G_DS + k) * n + i] = dS[k];
    }
#pragma unroll
    for (int k = 0; k < D * D; k++) p.grads[(G_V + k) * n + i] = gV[k];
  }
  if (!(mode & B_EOM)) return;
  double th[NTH];
#pragma unroll
  for (int q = 0; q < NTH; q++) th[q] = p.th[q * n + i];
  EomIn<D, R> in;
  in.th = th;
  in.it = p.clock->it;
  in.it2 = p.clock->it2;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    in.u[q] = (q < D) ? narrow<R>(p.y[(Y_U0 + q) * n + i]) : R(0);
    in.v[q] = va[q];
    in.gradP[q] = gP[q];
    in.gradBulk[q] = gB[q];
    in.gradshear[q] = gS[q];
    in.divshear[q] = dS[q];
  }
#pragma unroll
  for (int q = 0; q < 9; q++) in.gradV[q] = gV[q];
  in.g = narrow<R>(p.gam[i]);
  in.sigma = narrow<R>(p.sig[i]);
  in.sigma_lab = narrow<R>(p.slab[i]);
  in.m = narrow<R>(p.m[i]);
  in.Pi = narrow<R>(p.bulk[i]);
#pragma unroll
  for (int q = 0; q < NPI; q++) in.pi[q] = narrow<R>(p.pi[q * n + i]);
  const TransportT<R> k = transport<R>(rc.cfg, th);
  EomOut<R> o;
  DiffOut dout;
  if constexpr (DIFF) {
    DiffIn din;
    load_diff_in(rc, p, i, th, din);
    eom<D, R>(rc.cfg, k, in, t, o, nullptr, &din, &dout);
  } else {
    eom<D, R>(rc.cfg, k, in, t, o);
  }
  if (mode & B_DERIVS) {
#pragma unroll
    for (int q = 0; q < 3; q++) p.derivs[(D_DU0 + q) * n + i] = (q < D) ? double(o.du[q]) : 0.0;
    p.derivs[D_DS * n + i] = o.dS;
    p.derivs[D_DBULK * n + i] = o.dBulk;
#pragma unroll
    for (int q = 0; q < 5; q++) p.derivs[(D_DSHV0 + q) * n + i] = o.dShv[q];
    p.derivs[D_DEZ * n + i] = o.dEz;
    p.derivs[D_ETA * n + i] = k.eta;
    p.derivs[D_TAUPI * n + i] = k.tau_pi;
    p.derivs[D_ZETA * n + i] = k.zeta;
    p.derivs[D_TAUBULK * n + i] = k.tau_Pi;
    if constexpr (DIFF) {
#pragma unroll
      for (int c = 0; c < 3; c++) p.dif[(size_t)(F_DN + c) * n + i] = dout.dN[c];
#pragma unroll
      for (int q = 0; q < 9; q++) p.dif[(size_t)(F_DYQ + q) * n + i] = dout.dQ[q];
    }
  }
  if (!(mode & B_UPDATE)) return;
  const double* y0 = p.y0;
  double ynew[NY];
#pragma unroll
  for (int q = 0; q < NY; q++) ynew[q] = y0[q * n + i];
#pragma unroll
  for (int q = 0; q < D; q++) {
    ynew[Y_X0 + q] += dt_sub * p.v[q * n + i];
    ynew[Y_U0 + q] += dt_sub * widen<R>(o.du[q]);
  }
  double es = ynew[Y_ES] + dt_sub * widen<R>(o.dS);
  ynew[Y_EBULK] += dt_sub * widen<R>(o.dBulk);
#pragma unroll
  for (int q = 0; q < 5; q++) ynew[Y_SHV0 + q] += dt_sub * widen<R>(o.dShv[q]);
  ynew[Y_EZ] += dt_sub * widen<R>(o.dEz);
  double yq[9];
  if constexpr (DIFF) {
#pragma unroll
    for (int c = 0; c < 3; c++) ynew[Y_EB + c] += dt_sub * dout.dN[c];
#pragma unroll
    for (int q = 0; q < 9; q++) yq[q] = p.dif[(size_t)(F_YQ0 + q) * n + i] + dt_sub * dout.dQ[q];
  }
  if (es < 0.0) {
    if (p.freeze[i] > 3) es = 1.e-3;
    else flag_error(p.err, E_NEGS);
  }
  ynew[Y_ES] = es;
  bool finite = true;
#pragma unroll
  for (int q = 0; q < NY; q++) finite = finite && finite64(ynew[q]);
  if constexpr (DIFF) {
#pragma unroll
    for (int q = 0; q < 9; q++) finite = finite && finite64(yq[q]);
  }
  if (!finite) flag_error(p.err, E_NONFINITE);
#pragma unroll
  for (int q = 0; q < NY; q++) p.y[q * n + i] = ynew[q];
  if constexpr (DIFF) {
#pragma unroll
    for (int q = 0; q < 9; q++) p.dif[(size_t)(F_YQ + q) * n + i] = yq[q];
  }
  if (mode & B_WRITE_Y0) {
#pragma unroll
    for (int q = 0; q < NY; q++) p.y0[q * n + i] = ynew[q];
    if constexpr (DIFF) {
#pragma unroll
      for (int q = 0; q < 9; q++) p.dif[(size_t)(F_YQ0 + q) * n + i] = yq[q];
    }
  }
  const double x[3] = {ynew[Y_X0], ynew[Y_X1], D == 3 ? ynew[Y_X2] : 0.0};
  const double ext[4] = {ynew[Y_ES], ynew[Y_EB], ynew[Y_ESS], ynew[Y_EQ]};
  if constexpr (MIX) write_recAf<D>(p, i, x, p.m[i], ext);
  else write_recA<D>(p, i, x, p.m[i], ext);
}


// The device clock of one substep: substep 1 moves tau to t0 + dt/2 (the
// midpoint evaluation), substep 2 to t0 + dt, the start of the next step.
__device__ __forceinline__ void advance_clock(Clock* c, int substep, double dt) {
  if (substep == 1) c->t = c->teval = c->t0 + 0.5 * dt;
  else { c->t = c->t0 + dt; c->t0 = c->t; }
  c->it = 1.0 / c->t;
  c->it2 = 1.0 / (c->t * c->t);
}

// The freeze-out status machine of one particle after a step
// (FreezeOut::check_freeze_out_status, include/freeze_out.h:455-500, and the
// no-neighbour freeze of freeze_out_evo, :322-375): 0 fluid, 1 below e_FO,
// 3 freezing, 4 frozen.
__device__ __forceinline__ void freeze_particle(const RunConst& rc, const Ptrs& p, const int i) {
  if (i >= p.n) return;
  const int frzc = p.clock->frzc;
  const double ef = rc.efreeze;
  const double e = p.th[T_E * p.n + i];
  int f = p.freeze[i];
  if (f == 0) {
    if (e <= ef) f = 1;
  } else if (f == 1) {
    if (p.btrack[i] == -1) f = 3;
    else if (e > p.frz1_e[i]) f = 1;
    else if (e <= ef) f = 3;
    else f = 0;
  }
  if (frzc == 1) {
    p.frz1_e[i] = e;
    if (f == 3) f = 4;   // bsqsvinterpolate in the second step (:559-566)
  } else if (frzc >= 2) {
    if (f < 4 && p.btrack[i] == 0) {
      f = 4;
      p.btrack[i] = -1;
    }
    if (f == 3) f = 4;
    if (f < 4) p.frz1_e[i] = e;
  }
  p.freeze[i] = f;
}

}  // namespace passes
}  // namespace ccake
