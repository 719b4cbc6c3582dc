// Shared device definitions for the GB300 SPH hot path: state layout in HBM,
// the cubic-spline kernel, the neighbour-cell grid and run constants.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "ccake_gpu.h"

namespace ccake {

constexpr double kHbarcGeVfm = 0.1973269804;   // reference include/constants.h:16
constexpr double kHbarcMeVfm = 197.3269804;    // reference include/constants.h:17
constexpr double kTiny = 1e-25;                // reference include/eos_header.h:16
constexpr double kTbqsInf = 1e10;              // reference include/eos_header.h:17

// Evolved per-particle state (struct of arrays, one n-long slab per slot).
// The same layout is used for the current state Y and the step-start cache Y0.
enum YSlot : int {
  Y_X0 = 0, Y_X1, Y_X2,          // position (x, y, eta)
  Y_U0, Y_U1, Y_U2,              // spatial four-velocity u^i
  Y_ES, Y_EB, Y_ESS, Y_EQ,       // extensive s, rhoB, rhoS, rhoQ
  Y_EBULK,                       // extensive bulk pressure
  Y_SHV0, Y_SHV1, Y_SHV2, Y_SHV3, Y_SHV4,  // extensive pi^{ij}: (1,1)(1,2)(1,3)(2,2)(2,3)
  Y_EZ,                          // contribution_to_total_Ez
  NY
};

// Thermodynamic slots (the reference's thermo_info subset the path reads).
enum ThSlot : int { T_T = 0, T_MUB, T_MUS, T_MUQ, T_P, T_S, T_RB, T_RS, T_RQ, T_E, T_W, T_CS2,
                    T_DWDS, T_DWDB, T_DWDSS, T_DWDQ, NTH };  // dw/ds, dw/drhoB, dw/drhoS, dw/drhoQ

// Shear tensor pi^{mu nu} slots (upper triangle of the symmetric 4x4).
enum PiSlot : int { P00 = 0, P01, P02, P03, P11, P12, P13, P22, P23, P33, NPI };
__host__ __device__ constexpr int pi_slot(int i, int j) {
  return (i > j) ? pi_slot(j, i)
                 : (i == 0 ? j : (i == 1 ? 3 + j : (i == 2 ? 5 + j : 9)));
}

// Gradient slots written only when a caller asks for gradients.
enum GradSlot : int { G_P = 0, G_E = 3, G_B = 6, G_SH = 9, G_DS = 12, G_V = 15, NGRAD = 24 };

// Derivative slots written only when a caller asks for them.
enum DerivSlot : int { D_DU0 = 0, D_DU1, D_DU2, D_DS, D_DBULK, D_DSHV0, D_DSHV1, D_DSHV2, D_DSHV3,
                       D_DSHV4, D_DEZ, D_ETA, D_TAUPI, D_ZETA, D_TAUBULK,
                       // diagnostics of the last derivative evaluation (ccake_hydro_numbers):
                       // theta, sigma^{11,12,13,22,23}, shear / bulk Knudsen and inverse
                       // Reynolds numbers
                       D_THETA, D_SIG0, D_SIG1, D_SIG2, D_SIG3, D_SIG4, D_KNS, D_KNB, D_IRS, D_IRB,
                       D_SNU,   // shv_nabla_u = pi^{ij} nabla_i u_j of the last evaluation
                       NDER };

// Diffusion-sector slots (one n-long slab each; allocated only when the
// sector is on). Charges c = B, S, Q; spatial directions i = 0..2.
enum DifSlot : int {
  F_YQ = 0,     // 9: extensive q (3c + i), current state
  F_YQ0 = 9,    // 9: extensive q at the start of the RK2 step
  F_Q = 18,     // 12: q^mu (4c + mu) of the last evaluation (after the regulator)
  F_DA = 30,    // 12: dalpha_c/ds (c), dalpha_c/drho_d (3 + 3c + d)
  F_GQ = 42,    // 3: v . grad q^0 sums (grad_qa)
  F_DQ = 45,    // 3: div q (div_qa)
  F_GA = 48,    // 9: grad alpha (3i + c)
  F_DYQ = 57,   // 9: d(ext q)/dt (3c + i), written with the derivatives
  F_DN = 66,    // 3: d(ext rho)/dt, written with the derivatives
  F_KN = 69,    // 3: diffusion Knudsen numbers
  F_IR = 72,    // 3: diffusion inverse Reynolds numbers
  NDIF = 75
};
// Diffusion neighbour record (doubles): q^0_c / sl^2 (3), alpha_c (3),
// q^i_c / sl^2 at 6 + 3i + c (9), one pad.
constexpr int RQ = 16;

// Neighbour-record strides (doubles). Record A feeds the smoothing pass,
// record B the gradient pass; both are rewritten once per substep.
//   A: x0 x1 x2 m | m*ext_s m*ext_B m*ext_S m*ext_Q
//   B: x0 x1 x2 m | m*p/sl^2 m*e m*Pi/sl^2 0 | m*v^i (3) 0 | m*pi^{0i}/sl^2 (3) 0 |
//      m*pi^{ij}/sl^2 (11 12 13 22 23 33) 0 0
constexpr int RA = 8;
constexpr int RB = 24;
enum RecB : int { B_X0 = 0, B_X1, B_X2, B_M, B_P, B_E, B_PI, B_V0 = 8, B_PI0 = 12, B_PIJ = 16 };

// Neighbour-cell grid over a fixed box; cell edge >= 2h, indices clamped.
struct Grid {
  double lo[3];
  double inv_cs[3];
  int nc[3];
  int ncell;
};

// Run constants passed by value to every kernel.
// The cubic spline of one dimensionality and smoothing length in the forms
// the FP64 pair loop evaluates (the same member names as RunConst's own).
struct KernelConst {
  double inv_h, wn, wn2, gn, win_c1, win_c2, fin_a, fin_b;
};

struct RunConst {
  ccake_config cfg;
  Grid grid;
  double cut2;           // (2h)^2
  double cutc2;          // (2h + skin)^2, radius of the candidate list
  double inv_h;
  double wn, wn2;        // W normalisations knorm/h^D, knorm2/h^D
  double gn, gn2;        // grad W normalisations kgrad/h^(D+1), kgrad2/h^(D+1)
  double k0;             // W(0)
  // the cubic spline in the forms the FP64 pair loop evaluates:
  // W(q < 1) = wn + q^2 (win_c1 + win_c2 q), the grad-W factor for q < 1 is
  // fin_a q + fin_b
  double win_c1, win_c2, fin_a, fin_b;
  unsigned long long cut2_bits;   // IEEE bits of cut2 (for the integer-pipe predicate)
  // 3-D with the factorised kernel (src/kernel.cpp:129-170 of the reference):
  // W = W_2D(r_perp, hT) W_1D(|d eta|, hEta), the two factors' constants
  KernelConst kperp, keta;
  double efreeze;        // e(T_FO, 0, 0, 0)
  // FP32 copies for the FP32 pair loops, rounded once on the host (a
  // conversion in a kernel is an FP64-pipe instruction, and the compiler may
  // repeat it inside a loop rather than hold its result in a register)
  float fcut2, fcutc2, finv_h, fwn, fwn2, fgn, fgn2, fk0;
};

// Device-side clock: tau at the start of the RK2 step and the current tau.
struct Clock {
  double t0;
  double t;
  double teval;   // time of the last substep-2 derivative evaluation (t0 + dt/2)
  int32_t frzc;   // steps seen by the freeze-out status machine (0, 1, 2 = third and later)
  int32_t nstep;  // steps seen by the freeze-out stage (the step of a hypersurface row)
  double taup, taupp;   // times of the last two freeze-out snapshots (FreezeOut::taup, taupp)
  double it, it2;       // 1/t and 1/t^2 of the current t: one FP64 division a substep, not one a particle
};

// Freeze-out snapshot fields (FreezeOut::freeze_array, include/freeze_out.h):
// r[3] u[3] gradP[3] gradE[3] s e rhoB rhoS rhoQ T muB muS muQ theta bulk
// sigma_lab pi^{mu nu}[10 slots] pi^{33} shv_nabla_u w cs2 q^mu[3][4]; six snapshots
// (frz1 frz2 fback fback2 fback3 fback4), field q of particle i of snapshot k
// at (k * NSF + q) * n + i.
enum SnapField : int { SF_R = 0, SF_U = 3, SF_GP = 6, SF_GE = 9, SF_S = 12, SF_E, SF_RB, SF_RS, SF_RQ, SF_T, SF_MUB,
                       SF_MUS, SF_MUQ, SF_THETA, SF_BULK, SF_SLAB, SF_SHV, SF_SHV33 = SF_SHV + 10, SF_SNU, SF_W, SF_CS2,
                       SF_Q, NSF = SF_Q + 12 };
// a freeze_out.dat row on the device: step, particle, then the fields
// (src/output.cpp:433-475), 40 in 2-D, 45 in 3-D
constexpr int kFoRow = 2 + 45;

// Error counters raised by the kernels (read back by the host after a call).
// E_FIRST holds 1 + the slot of the first failure raised since the counters
// were cleared, so that the host reports the failure that happened first:
// the reference aborts at its first failure, and later ones (an EoS failure
// at a particle whose entropy went negative a substep earlier) follow from it.
enum ErrSlot : int { E_EOS = 0, E_NEGS = 1, E_NONFINITE = 2, E_NBR_OVERFLOW = 3, E_FIRST = 4, NERR = 5 };

#ifdef __CUDACC__
__device__ __forceinline__ void flag_error(int32_t* err, int slot) {
  atomicAdd(&err[slot], 1);
  atomicCAS(&err[E_FIRST], 0, slot + 1);
}
#endif

// Kernel normalisations of the reference, src/kernel.cpp:11-26.
__host__ __device__ inline double knorm(int D) { return D == 1 ? 2. / 3. : D == 2 ? 10. / (7 * M_PI) : 1. / M_PI; }
__host__ __device__ inline double knorm2(int D) { return D == 1 ? 1. / 6. : D == 2 ? 5. / (14. * M_PI) : 1. / (4 * M_PI); }
__host__ __device__ inline double kgrad(int D) { return D == 1 ? -1. / 2. : D == 2 ? -15. / (14. * M_PI) : -3. / (4. * M_PI); }
__host__ __device__ inline double kgrad2(int D) { return D == 1 ? 1. : D == 2 ? 15. / (7. * M_PI) : 3. / (2. * M_PI); }

// FP64 <-> FP32 conversions and the FP64 finiteness test on the integer pipe
// (device; plain casts on the host). A hardware conversion issues to the
// FP64 pipe, the narrowest unit of this GPU -- in the mixed-form kernels the
// conversions kept it busier than their FP64 arithmetic did -- while the
// integer pipe has room to spare. Both follow the IEEE 754 binary32 and
// binary64 formats: narrowing rounds to nearest, ties to even, for
// magnitudes in the normal FP32 range (the bits a hardware conversion gives
// there), gives signed zero below that range and infinity above it, and
// keeps NaN; widening is exact for normal FP32 values, zeros, infinities and
// NaN, and flushes FP32 subnormals to signed zero.
__host__ __device__ __forceinline__ float f32_rn(double x) {
#ifdef __CUDA_ARCH__
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned s = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long m = b & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long t = m - (896ull << 52);   // exponent bias 1023 -> 127
  const unsigned long long r = (t + 0x0FFFFFFFull + ((t >> 29) & 1ull)) >> 29;
  unsigned f = r >= 0x7F800000ull ? 0x7F800000u : (unsigned)r;
  if (m < (897ull << 52)) f = 0u;
  if (m >= 0x7FF0000000000000ull) f = m == 0x7FF0000000000000ull ? 0x7F800000u : 0x7FC00000u;
  return __uint_as_float(s | f);
#else
  return (float)x;
#endif
}

__host__ __device__ __forceinline__ double f64_of(float v) {
#ifdef __CUDA_ARCH__
  const unsigned b = __float_as_uint(v);
  const unsigned s = b & 0x80000000u, m = b & 0x7FFFFFFFu;
  unsigned hi = s | ((m >> 3) + (896u << 20));   // exponent bias 127 -> 1023
  if (m >= 0x7F800000u) hi = s | 0x7FF00000u | ((m & 0x007FFFFFu) >> 3);
  if (m < 0x00800000u) hi = s;
  const unsigned lo = m < 0x00800000u ? 0u : (m << 29);
  return __hiloint2double((int)hi, (int)lo);
#else
  return (double)v;
#endif
}

__host__ __device__ __forceinline__ bool finite64(double x) {
#ifdef __CUDA_ARCH__
  return (__double2hiint(x) & 0x7FF00000) != 0x7FF00000;
#else
  return std::isfinite(x);
#endif
}

// R(x) for the arithmetic type R of a templated kernel body (FP64 or FP32),
// and back, by the conversions above.
template <typename R>
__host__ __device__ __forceinline__ R narrow(double x) {
  if constexpr (sizeof(R) == sizeof(float)) return f32_rn(x);
  else return x;
}
template <typename R>
__host__ __device__ __forceinline__ double widen(R x) {
  if constexpr (sizeof(R) == sizeof(float)) return f64_of(x);
  else return x;
}

// Constants of the D-dimensional spline with smoothing length h (host).
inline KernelConst kernel_const(int D, double h) {
  KernelConst k;
  k.inv_h = 1.0 / h;
  k.wn = knorm(D) / std::pow(h, D);
  k.wn2 = knorm2(D) / std::pow(h, D);
  k.gn = kgrad(D) / std::pow(h, D + 1);
  const double gn2 = kgrad2(D) / std::pow(h, D + 1);
  k.win_c1 = -1.5 * k.wn;
  k.win_c2 = 0.75 * k.wn;
  k.fin_a = 1.5 * gn2 * k.inv_h;
  k.fin_b = -2.0 * gn2 * k.inv_h;
  return k;
}

// Kernel constants of a run with smoothing length h in D dimensions (host).
inline void set_kernel_constants(RunConst& rc, int D, double h) {
  rc.cut2 = (2.0 * h) * (2.0 * h);
  std::memcpy(&rc.cut2_bits, &rc.cut2, sizeof(double));
  rc.inv_h = 1.0 / h;
  rc.wn = knorm(D) / std::pow(h, D);
  rc.wn2 = knorm2(D) / std::pow(h, D);
  rc.gn = kgrad(D) / std::pow(h, D + 1);
  rc.gn2 = kgrad2(D) / std::pow(h, D + 1);
  rc.k0 = rc.wn;   // W(0)
  rc.win_c1 = -1.5 * rc.wn;
  rc.win_c2 = 0.75 * rc.wn;
  rc.fin_a = 1.5 * rc.gn2 * rc.inv_h;
  rc.fin_b = -2.0 * rc.gn2 * rc.inv_h;
  rc.fcut2 = (float)rc.cut2;
  rc.finv_h = (float)rc.inv_h;
  rc.fwn = (float)rc.wn;
  rc.fwn2 = (float)rc.wn2;
  rc.fgn = (float)rc.gn;
  rc.fgn2 = (float)rc.gn2;
  rc.fk0 = (float)rc.k0;
}

// Exact squared distance of the neighbour predicate (reference Cabana
// VerletList, cutoff 2h): products and sums rounded separately, no FMA.
template <int D>
__device__ __forceinline__ double dist2_exact(const double* d) {
  double s = __dmul_rn(d[0], d[0]);
  s = __dadd_rn(s, __dmul_rn(d[1], d[1]));
  if (D == 3) s = __dadd_rn(s, __dmul_rn(d[2], d[2]));
  return s;
}

// Cell coordinate of a position along one axis, clamped to the grid.
__device__ __forceinline__ int cell_coord(const Grid& g, int k, double x) {
  int c = (int)floor((x - g.lo[k]) * g.inv_cs[k]);
  return c < 0 ? 0 : (c >= g.nc[k] ? g.nc[k] - 1 : c);
}

}  // namespace ccake
