// Device per-particle physics of the hot path: transport coefficients, the
// pi^{mu nu} constraints, and the MRF equations of motion (ideal + shear +
// bulk + diffusion, Milne and Cartesian coordinates) for one particle.
// Templated on dimension and on the arithmetic type (FP64, or FP32 for the
// mixed form, which has no diffusion sector).
#pragma once
#include <type_traits>

#include "common.cuh"

namespace ccake {

template <typename R = double>
struct TransportT {
  R eta, tau_pi, zeta, tau_Pi, delta_PiPi, delta_pipi, lambda_piPi, lambda_Pipi, phi1, phi3, phi6, phi7, tau_pipi;
};
using Transport = TransportT<double>;

// x^p; integer exponents 0..8 by repeated products (exact to rounding, and
// a fraction of pow's instruction count), others by pow.
template <typename R>
__device__ __forceinline__ R powi_or_pow(R x, R p) {
  if (p == R(2)) return x * x;
  if (p >= R(0) && p <= R(8) && p == floor(p)) {
    R r = R(1);
    for (int k = 0; k < (int)p; k++) r *= x;
    return r;
  }
  return pow(x, p);
}

// Reference src/transport_coefficients.cpp:620-900 (modes used by the hot
// path). R = double for the plain form; R = float where the coefficients only
// feed the mixed form's FP32 equations of motion.
template <typename R = double>
__device__ inline TransportT<R> transport(const ccake_config& c, const double* th) {
  TransportT<R> k;
  const R T = narrow<R>(th[T_T]), w = narrow<R>(th[T_W]), cs2 = narrow<R>(th[T_CS2]), p = narrow<R>(th[T_P]);
  const R eos = R(c.eta_over_s), zos = R(c.zeta_over_s), zp = R(c.zeta_cs2_p);
  const R k13 = R(1.0) / R(3.0);
  k.eta = (T <= R(0)) ? R(0) : eos * (w / T);
  if (c.shear_relax_mode == 1) k.tau_pi = (R(5) * k.eta) / w;
  else if (c.shear_relax_mode == 2) k.tau_pi = fmax((R(5) * k.eta) / w, R(0.001));
  else k.tau_pi = fmax(R(5) * k.eta / w, R(0.005));
  switch (c.zeta_mode) {
    case 1: k.zeta = zos * (w / T); break;
    case 2: {
      R factor = R(1);
      if (c.modulate_zeta_with_tanh) {
        const R Ttr = R(150.0 / kHbarcMeVfm), Tsc = R(10.0 / kHbarcMeVfm);
        const R thx = tanh((T - Ttr) / Tsc), xp = powi_or_pow<R>(T / Ttr, zp);
        factor = R(0.5) * (R(1) + xp) + R(0.5) * (R(1) - xp) * thx;
      }
      k.zeta = R(c.zeta_cs2_A) * factor * powi_or_pow<R>(k13 - fmin(cs2, R(1)), zp) * w / T;
      break;
    }
    case 3: {
      const R x = (T - R(c.zeta_peak_T)) / R(c.zeta_peak_width);
      k.zeta = zos * exp(R(-0.5) * x * x) * (w / T);
      break;
    }
    default: k.zeta = R(0.005) * (w / T);
  }
  const R cc = cs2 > R(1) ? R(1) : cs2;
  const R pw = powi_or_pow<R>(k13 - cc, zp);
  k.tau_Pi = (pw < R(1e-10)) ? R(1e10) : fmax(R(5) * k.zeta / (pw * w), R(0.1));
  // second-order coefficients by mode (src/transport_coefficients.cpp:
  // 380-560 switches, :704-912 the functions): 0 the *_DEFAULT function,
  // 1 israel-stewart (the two deltas), 2 disabled. phi1, phi3 and phi6 are 0
  // in every mode.
  auto pick = [](int32_t mode, R def, R is) { return mode == 2 ? R(0) : (mode == 1 ? is : def); };
  k.delta_PiPi = pick(c.delta_PiPi_mode, R(2) * k.tau_Pi / R(3), k.tau_Pi);
  k.delta_pipi = pick(c.delta_pipi_mode, R(4) * k.tau_pi / R(3), k.tau_pi);
  k.lambda_piPi = pick(c.lambda_piPi_mode, R(6) / R(5) * k.tau_pi, R(0));
  k.lambda_Pipi = pick(c.lambda_Pipi_mode, R(8) * (k13 - cc) * k.tau_Pi / R(5), R(0));
  k.phi1 = R(0);
  k.phi3 = R(0);
  k.phi6 = R(0);
  k.phi7 = pick(c.phi7_mode, R(9) / (R(70) * p), R(0));
  k.tau_pipi = pick(c.tau_pipi_mode, R(10) * k.tau_pi / R(7), R(0));
  return k;
}

// Diffusion coefficients, src/transport_coefficients.cpp:571-617 (kappa,
// tauq), :918-973 (default_kappa = kappa/T^2 T^2, default_tauq = 0.2/T on
// the diagonal), :981-1040 (kappaB_coth, tauqB_only) and :1048-1057 (the
// Gaussian suppression near the critical point, table EoS only). tq, kq
// row-major 3x3 over (B, S, Q).
__device__ inline void diffusion_coefs(const ccake_config& c, const double* th, bool table_eos, double* tq,
                                       double* kq) {
  const double T = th[T_T];
  for (int k = 0; k < 9; k++) tq[k] = kq[k] = 0.0;
  if (c.diffusion_mode == 2) {
    const double muB = th[T_MUB], nB = th[T_RB], w = th[T_W];
    const double x = (T > kTiny) ? muB / T : 0.0;
    if (T > kTiny && fabs(w) > kTiny && fabs(x) > 1.0e-2) {
      const double kB = (c.C_B / T) * nB * ((1.0 / 3.0) / tanh(x) - nB * T / w);
      if (isfinite(kB) && kB > 0.0) kq[0] = kB;
    }
    if (c.diffusion_relax_mode == 1) {
      if (T > kTiny)
        for (int i = 0; i < 3; i++) tq[4 * i] = c.C_B / T;
    } else {
      for (int i = 0; i < 3; i++) tq[4 * i] += 0.2 / T;
    }
    return;
  }
  double sup = 1.0;
  if (c.critical_scaling_diffusion && table_eos) {
    const double dT = T - c.crit_T / kHbarcMeVfm, dm = th[T_MUB] - c.crit_muB / kHbarcMeVfm;
    const double sT = c.crit_wT / kHbarcMeVfm, sm = c.crit_wmuB / kHbarcMeVfm;
    const double ex = 0.5 * (dT * dT / (sT * sT) + dm * dm / (sm * sm));
    sup = 1.0 - exp(-ex);
  }
  for (int k = 0; k < 9; k++) kq[k] = sup * c.kappa_over_T2[k] * (T * T);
  for (int i = 0; i < 3; i++) tq[4 * i] += 0.2 / T;
}

// 3x3 inverse by cofactors over the determinant (include/milne.hpp:788-834),
// the cofactors times one reciprocal of the determinant.
template <typename R>
__device__ inline void inverse3(const R* A, R* Ai) {
#define M3(i, j) A[(i) * 3 + (j)]
  const R det = M3(0, 0) * M3(1, 1) * M3(2, 2) + M3(0, 1) * M3(1, 2) * M3(2, 0) + M3(0, 2) * M3(1, 0) * M3(2, 1) -
                M3(0, 2) * M3(1, 1) * M3(2, 0) - M3(0, 1) * M3(1, 0) * M3(2, 2) - M3(0, 0) * M3(1, 2) * M3(2, 1);
  const R id = R(1.0) / det;
  Ai[0] = (M3(1, 1) * M3(2, 2) - M3(1, 2) * M3(2, 1)) * id;
  Ai[1] = (M3(0, 2) * M3(2, 1) - M3(0, 1) * M3(2, 2)) * id;
  Ai[2] = (M3(0, 1) * M3(1, 2) - M3(0, 2) * M3(1, 1)) * id;
  Ai[3] = (M3(1, 2) * M3(2, 0) - M3(1, 0) * M3(2, 2)) * id;
  Ai[4] = (M3(0, 0) * M3(2, 2) - M3(0, 2) * M3(2, 0)) * id;
  Ai[5] = (M3(0, 2) * M3(1, 0) - M3(0, 0) * M3(1, 2)) * id;
  Ai[6] = (M3(1, 0) * M3(2, 1) - M3(1, 1) * M3(2, 0)) * id;
  Ai[7] = (M3(0, 1) * M3(2, 0) - M3(0, 0) * M3(2, 1)) * id;
  Ai[8] = (M3(0, 0) * M3(1, 1) - M3(0, 1) * M3(1, 0)) * id;
#undef M3
}

// Diffusion inputs of the equations of motion for one particle (FP64 form).
struct DiffIn {
  double q[12];          // q^mu of charge c at 4c + mu
  double da[12];         // dalpha_c/ds (c), dalpha_c/drho_d (3 + 3c + d)
  double ga[9];          // grad alpha, direction i, charge c at 3i + c (i < D)
  double gq[3], dq[3];   // v . grad q^0 and div q sums
  double tq[9], kq[9];   // tau_q, kappa_q
};
struct DiffOut {
  double dN[3];          // d(ext rho_c)/dt
  double dQ[9];          // d(ext q)/dt, charge c, direction i at 3c + i
};

// gamma = sqrt(1 - u_i u^i) in Milne coordinates (reference src/eom_default.cpp:17-38,
// include/milne.hpp:92-96 and :354).
template <int D>
__device__ __forceinline__ double gamma_milne(const double* u, double t2) {
  double c = u[0] * u[0] + u[1] * u[1];
  if (D == 3) c += t2 * u[2] * u[2];
  return sqrt(1.0 + c);
}

// pi^{mu nu} from the extensive spatial components, tracelessness and
// orthogonality (reference src/eom_default.cpp:56-172). pi[] uses PiSlot.
// In 2-D the eta velocity is zero and its terms are left out (the same
// values; a product with a constant zero would still cost FP64 instructions).
template <int D>
__device__ inline void reset_pi(const double* ext_shv, double sigma, double g, const double* u3, double t2,
                                double it2, double* pi) {
  const double f0 = -u3[0], f1 = -u3[1], f2 = -t2 * u3[2];   // covariant u_i
  const double p11 = ext_shv[0] * sigma, p12 = ext_shv[1] * sigma, p13 = ext_shv[2] * sigma;
  const double p22 = ext_shv[3] * sigma, p23 = ext_shv[4] * sigma;
  // one division for 1/g (FP64 division is a long sequence); it2 = 1/t^2
  const double ig = 1.0 / g;
  double p00;
  if (D == 3)
    p00 = (f0 * f0 * p11 + f1 * f1 * p22 + 2. * f1 * f0 * p12 + 2. * f2 * f0 * p13 + 2. * f2 * f1 * p23 -
           f2 * f2 * (p11 + p22) * it2) / (g * g - f2 * f2 * it2);
  else
    p00 = (f0 * f0 * p11 + f1 * f1 * p22 + 2. * f1 * f0 * p12) / (g * g);
  const double p33 = (p00 - p11 - p22) * it2;
  pi[P00] = p00; pi[P11] = p11; pi[P12] = p12; pi[P13] = p13; pi[P22] = p22; pi[P23] = p23; pi[P33] = p33;
  if (D == 3) {
    pi[P01] = -(p11 * f0 + p12 * f1 + p13 * f2) * ig;
    pi[P02] = -(p12 * f0 + p22 * f1 + p23 * f2) * ig;
    pi[P03] = -(p13 * f0 + p23 * f1 + p33 * f2) * ig;
  } else {
    pi[P01] = -(p11 * f0 + p12 * f1) * ig;
    pi[P02] = -(p12 * f0 + p22 * f1) * ig;
    pi[P03] = -(p13 * f0 + p23 * f1) * ig;
  }
}

// Inputs of the equations of motion for one particle.
template <int D, typename R = double>
struct EomIn {
  R u[3], v[3];
  R g, sigma, sigma_lab, m;
  double it, it2;            // 1/t and 1/t^2 at the evaluation time (FP64)
  const double* th;          // NTH thermo values (FP64, from the EoS)
  R Pi;                      // bulk pressure
  R pi[NPI];                 // pi^{mu nu}
  R gradP[3], gradBulk[3], gradshear[3], divshear[3], gradV[9];
};

template <typename R = double>
struct EomOut {
  R du[3], dS, dBulk, dShv[5], dEz;
};

// Reference src/eom_default.cpp:211-869 (evaluate_time_derivatives) and
// :882-1412 (calculate_MRF_shear), without sources, for one particle at time t.
// R = double is the plain FP64 form; R = float is the mixed form's EoM (the
// state update it feeds stays FP64).
// diag (optional, 7 values): theta, sigma^{11,12,13,22,23} and
// shv_nabla_u (src/eom_default.cpp:764-807); the hot kernels pass none.
// dif / dout (FP64 form only): the diffusion sector, src/eom_default.cpp:
// 1415-1817 (calculate_MRF_diffusion; the stray semicolon of :1744 ends
// F_D_ib after its second term), :368-451 (charge MRFs), :579-617 (coupling
// into du/dt), :690-736 (dN/dt, d(ext q)/dt) and the R_S dN/dt entropy term.
template <int D, typename R = double>
__device__ inline void eom(const ccake_config& cfg, const TransportT<R>& k, const EomIn<D, R>& in, double td,
                           EomOut<R>& o, R* diag = nullptr, const DiffIn* dif = nullptr, DiffOut* dout = nullptr) {
  R sigF[5] = {0, 0, 0, 0, 0}, sigM[5][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  const R t = narrow<R>(td);
  // Cartesian coordinates (coord = 1, src/eom_cartesian.cpp:210-1400): the
  // metric without tau (tm = 1) and none of the Milne connection terms (1/tau
  // sources, the geometric factor, the eta deltas; ch = 0, itc = 0)
  const bool cart = cfg.coord == 1;
  const R tm = cart ? R(1.0) : t, ch = cart ? R(0.0) : R(1.0);
  const R t2 = tm * tm;
  const R g = in.g, sig = in.sigma;
  // reciprocals: FP64 division is a long instruction sequence on the scarce
  // FP64 pipe, so each divisor is inverted once
  // the FP64 form takes 1/t and 1/t^2 from the clock (the same values; one
  // division a substep instead of two a particle)
  constexpr bool f64 = sizeof(R) == sizeof(double);
  const R ig = R(1.0) / g, it = f64 ? R(in.it) : R(1.0) / t;
  const R it2 = cart ? R(1.0) : (f64 ? R(in.it2) : R(1.0) / t2);
  const R itc = cart ? R(0.0) : it, itm = cart ? R(1.0) : it;
  const R k13 = R(1.0) / R(3.0), k16 = R(1.0) / R(6.0);
  const double* th = in.th;
  const R T = narrow<R>(th[T_T]), w = narrow<R>(th[T_W]), sden = narrow<R>(th[T_S]), dwds = narrow<R>(th[T_DWDS]);
  const R rho[3] = {narrow<R>(th[T_RB]), narrow<R>(th[T_RS]), narrow<R>(th[T_RQ])};
  const R dwdr[3] = {narrow<R>(th[T_DWDB]), narrow<R>(th[T_DWDSS]), narrow<R>(th[T_DWDQ])};
  const R Pi = in.Pi;
  auto P = [&](int i, int j) { return in.pi[pi_slot(i, j)]; };
  // covariant spatial velocity (Vector<D>::make_covariant)
  R u[3] = {in.u[0], in.u[1], D == 3 ? in.u[2] : R(0.0)};
  R uc[3] = {-u[0], -u[1], D == 3 ? -t2 * u[2] : R(0.0)};
  R divV = R(0.0);
#pragma unroll
  for (int i = 0; i < D; i++) divV += in.gradV[i * D + i];
  const R uD = u[D - 1];
  const R geo = (D == 3 && !cart) ? uD * uD * t * ig : R(0.0);
  // In 2-D the geometric term geo, every eta delta dEta(i) and the eta
  // velocity vanish. A product with a constant zero is still an FP64
  // instruction (IEEE arithmetic keeps NaN and the sign of zero), and the
  // FP64 pipe bounds this function, so those terms are left out at compile
  // time (if (D == 3) / if (e3) below): the results are the same up to the
  // sign of zero.
  constexpr bool e3 = (D == 3);
  R expn = g * divV + g * itc;
  if (e3) expn = expn + geo;
  auto dEta = [cart](int i) { return (!cart && D == 3 && i == 2) ? R(1.0) : R(0.0); };

  // ---- shear MRFs --------------------------------------------------------
  R M0i[9] = {0}, F0i[3] = {0}, Mnab[3] = {0}, Fnab = R(0.0);
  R Mext[5][3] = {{0}}, Fext[5] = {0};
  R ss = R(0.0);   // pi^{mu nu} pi_{mu nu}
  if (cfg.using_shear) {
    const R cmd[4] = {R(1.0), -R(1.0), -R(1.0), -R(1.0) * itm * itm};
    const R eta = k.eta, phi7 = k.phi7, lpP = k.lambda_piPi;
    const R tpp = k.tau_pipi, dpp = k.delta_pipi, tpi = k.tau_pi;
    const R tdelta = dpp - tpi;
    const R itg = R(1.0) / (tpi * g), istg = R(1.0) / (sig * tpi * g);
    const R v[3] = {in.v[0], in.v[1], D == 3 ? in.v[2] : R(0.0)};
    const R fu[3] = {u[0], u[1], u[2]};
    const R fuc[3] = {-u[0], -u[1], -t2 * u[2]};
    R pi[4][4], hy[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
        pi[i][j] = P(i, j);
        hy[i][j] = pi[i][j] * ((j == 1 || j == 2) ? -R(1.0) : (j == 3 ? -t2 : R(1.0)));   // pi^mu_nu
      }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) ss += pi[i][j] * hy[i][j] * ((i == 1 || i == 2) ? -R(1.0) : (i == 3 ? -t2 : R(1.0)));
    R gu[3][3] = {{0}}, gu0[3] = {0}, cgu[3][3] = {{0}};
#pragma unroll
    for (int i = 0; i < D; i++)
#pragma unroll
      for (int j = 0; j < D; j++) {
        R acc = g * in.gradV[i * D + j];
#pragma unroll
        for (int kk = 0; kk < D; kk++) acc += -g * u[j] * uc[kk] * in.gradV[i * D + kk];
        gu[i][j] = acc;
      }
#pragma unroll
    for (int i = 0; i < D; i++) {
      R acc = 0;
#pragma unroll
      for (int j = 0; j < D; j++) acc += gu[i][j] * uc[j];
      gu0[i] = -R(1.) * acc * ig;
#pragma unroll
      for (int j = 0; j < D; j++) cgu[i][j] = gu[i][j] * ((D == 2 || i < D - 1) ? -R(1.0) : -R(1.0) * it2);
    }
    R gu0c[3] = {-gu0[0], -gu0[1], D == 3 ? -gu0[2] * it2 : R(0.0)};
    R guv[3] = {0, 0, 0}, gu0v = R(0.0);
#pragma unroll
    for (int j = 0; j < D; j++) {
#pragma unroll
      for (int kk = 0; kk < D; kk++) guv[j] += gu[kk][j] * v[kk];
      gu0v += gu0[j] * v[j];
    }
    R vgs[3], ggs[3], sgu[3], vsg[3], sl0[3];
    R sgu_s = R(0.0);
#pragma unroll
    for (int i = 0; i < D; i++) {
      R a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0;
#pragma unroll
      for (int j = 0; j < D; j++) {
        a1 += guv[j] * hy[i + 1][j + 1];
        a2 += cgu[i][j] * hy[0][j + 1];
        a3 += pi[j + 1][0] * gu[j][i] + pi[j + 1][i + 1] * gu0[j];
        a4 += v[j] * pi[0][0] * gu[j][i] + v[j] * pi[0][i + 1] * gu0[j];
        sgu_s += (hy[i + 1][j + 1] - v[i] * hy[0][j + 1]) * gu[i][j];
      }
      sgu_s += (hy[i + 1][0] - v[i] * hy[0][0]) * gu0[i];
      vgs[i] = a1 + gu0v * hy[i + 1][0];
      ggs[i] = a2 + cmd[i + 1] * gu0[i] * hy[0][0];
      sgu[i] = a3;
      vsg[i] = a4;
#pragma unroll
      for (int j = 0; j < 4; j++) a5 += (pi[0][j] * hy[i + 1][j] + pi[i + 1][j] * hy[0][j]) / R(2.);
      sl0[i] = a5;
    }
    // four-acceleration MRFs
    const R uv = cfg.using_vorticity ? R(1.0) : R(0.0);
#pragma unroll
    for (int i = 0; i < D; i++) {
      const R di = dEta(i);
      R Fs, FD = R(0.0), Fds, Fdo;
      if (e3) {
        Fs = -(guv[i] - gu0c[i]) / R(2.) + u[i] * g * expn * k13 - g * geo * u[i] / R(2.);
        FD = g * (u[i] * hy[0][0] + g * hy[i + 1][0]) * geo + t * uD * pi[3][i + 1] * di;
        Fds = -(vgs[i] - ggs[i] - R(4.) * g * u[i] * sgu_s * k13 - sgu[i] + vsg[i]) / R(4.) +
              (hy[i + 1][0] - g * g * hy[i + 1][0] - g * u[i] * hy[0][0] + pi[0][i + 1] +
               R(4.) * u[i] * g * hy[0][0] * k13) * geo / R(4.) +
              ch * ((g * cmd[i + 1] * hy[0][3] * di * it + g * pi[3][0] * di * it + R(4.) * g * u[i] * (g * hy[3][3] * it) * k13) / R(4.)) -
              pi[0][i + 1] * (g * itc + geo + g * divV) * k13;
        Fdo = -(vgs[i] - ggs[i] + sgu[i] - vsg[i]) / R(4.) +
              (hy[i + 1][0] - g * g * hy[i + 1][0] - g * u[i] * hy[0][0] - pi[0][i + 1]) * geo / R(4.) +
              (g * cmd[i + 1] * hy[0][3] * di * it - g * pi[3][0] * di * it) / R(4.);
        Fs += di * (-(-uD * t - uD * it + g * uD * uD * t + R(2.) * g * g * uD * it) / R(2.));
        FD += di * (uD * pi[0][0] * it + g * pi[3][0] * it);
      } else {
        Fs = -(guv[i] - gu0c[i]) / R(2.) + u[i] * g * expn * k13;
        Fds = -(vgs[i] - ggs[i] - R(4.) * g * u[i] * sgu_s * k13 - sgu[i] + vsg[i]) / R(4.) +
              ch * ((R(4.) * g * u[i] * (g * hy[3][3] * it) * k13) / R(4.)) - pi[0][i + 1] * (g * itc + g * divV) * k13;
        Fdo = -(vgs[i] - ggs[i] + sgu[i] - vsg[i]) / R(4.);
      }
      const R Fdd = pi[i + 1][0] * expn;
      if (D == 3 && !cart) {
        Fds += (t * uD * di * cmd[i + 1] * hy[0][0] + uD * hy[i + 1][3] * g * it / R(4.) + hy[i + 1][3] * t * uD +
                pi[0][0] * di * uD * it + t * uD * uD * (g * hy[i + 1][0] + u[i] * hy[0][0]) +
                R(2.) * g * uD * (g * hy[i + 1][3] + u[i] * pi[0][3]) * it) / R(4.) +
               g * u[i] * (hy[3][0] * uD * t + uD * hy[0][3] * it) * k13;
        Fdo += (t * uD * di * cmd[i + 1] * hy[0][0] + uD * hy[i + 1][3] * g * it - hy[3][i + 1] * t * uD -
                pi[0][0] * di * uD * it + t * uD * uD * (g * hy[i + 1][0] + u[i] * hy[0][0]) +
                R(2.) * g * uD * (g * hy[i + 1][3] + u[i] * pi[0][3]) * it) / R(4.);
      }
      // phi6 (and phi1, phi3 below) are zero in every coefficient mode:
      // their terms are left out
      R f0 = -pi[i + 1][0];
      if (e3) f0 = f0 - tpi * FD;
      F0i[i] = (f0 - dpp * Fdd + R(2.) * tpi * Fdo * uv - tpp * Fds + (R(2.) * eta + lpP * Pi) * Fs +
                phi7 * (sl0[i] + g * u[i] * ss * k13)) * itg;
#pragma unroll
      for (int j = 0; j < D; j++) {
        R Ms = u[i] * uc[j] * k16;
        const R MD = g * u[i] * (hy[0][j + 1] - hy[0][0] * uc[j] * ig) + g * g * (hy[i + 1][j + 1] - hy[i + 1][0] * uc[j] * ig);
        R Mds = (hy[i + 1][j + 1] - hy[i + 1][0] * uc[j] * ig - g * g * hy[i + 1][j + 1] - g * u[i] * hy[0][j + 1] +
                      uc[j] * g * hy[i + 1][0] + uc[j] * u[i] * hy[0][0] +
                      R(4.) * g * u[i] * (hy[0][j + 1] - hy[0][0] * uc[j] * ig) * k13 +
                      (-pi[0][i + 1] + R(4.) * pi[0][i + 1] * k13) * uc[j] * ig) / R(4.);
        R Mdo = (hy[i + 1][j + 1] - hy[i + 1][0] * uc[j] * ig - g * g * hy[i + 1][j + 1] - g * u[i] * hy[0][j + 1] +
                      uc[j] * g * hy[i + 1][0] + uc[j] * u[i] * hy[0][0] + pi[0][i + 1] * uc[j] * ig) / R(4.);
        const R Mdd = -pi[i + 1][0] * uc[j] * ig;
        if (i == j) {
          Ms += (R(1.) - g * g) / R(2.);
          Mdo += -pi[0][0] / R(4.);
          Mds += +pi[0][0] / R(4.);
        }
        M0i[i * D + j] = (-tpi * MD - dpp * Mdd + R(2.) * tpi * Mdo * uv - tpp * Mds + (R(2.) * eta + lpP * Pi) * Ms) * itg;
      }
    }
    // pi^{ij} nabla_i u_j MRF
#pragma unroll
    for (int i = 0; i < D; i++) {
      Mnab[i] = hy[0][i + 1] - hy[0][0] * uc[i] * ig;
#pragma unroll
      for (int j = 0; j < D; j++) Fnab += (hy[i + 1][j + 1] - v[i] * hy[0][j + 1]) * gu[i][j];
      Fnab += (hy[i + 1][0] - v[i] * hy[0][0]) * gu0[i];
    }
    if (e3) Fnab += +ch * (hy[3][3] * g * it) + hy[0][0] * geo + (t * hy[3][0] + hy[0][3] * it) * uD * dEta(D - 1);
    else Fnab += ch * (hy[3][3] * g * it);
    // shear-tensor evolution MRFs on the (i <= j) entries of the 2x3 block
    const R f2 = fu[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
#pragma unroll
      for (int j = i; j < 3; j++) {
        const int slot = (i == 0) ? j : 2 + j;   // (0,0)(0,1)(0,2)(1,1)(1,2) -> 0..4
        const R di = dEta(i), dj = dEta(j);
        R gugjs = 0, sigu = 0, vsig = 0, sml = 0;
#pragma unroll
        for (int kk = 0; kk < D; kk++) {
          const R cg_i = (i < D) ? cgu[i][kk] : R(0.0), cg_j = (j < D) ? cgu[j][kk] : R(0.0);
          const R g3_j = (kk < D && j < D) ? gu[kk][j] : R(0.0), g3_i = (i < D) ? gu[kk][i] : R(0.0);
          gugjs += cg_i * hy[j + 1][kk + 1] + cg_j * hy[i + 1][kk + 1];
          sigu += pi[kk + 1][i + 1] * g3_j + pi[kk + 1][j + 1] * g3_i;
          vsig += v[kk] * pi[0][i + 1] * g3_j + v[kk] * pi[0][j + 1] * g3_i;
        }
#pragma unroll
        for (int kk = 0; kk < 4; kk++) sml += (pi[i + 1][kk] * hy[j + 1][kk] + pi[j + 1][kk] * hy[i + 1][kk]) / R(2.);
        // in 2-D the eta row (j = 2) has fu[j] = 0
        const bool fj0 = (D == 2 && j == 2);
        R FD2 = R(0.0);
        if (e3) FD2 = g * geo * (fu[i] * hy[j + 1][0] + fu[j] * hy[i + 1][0]);
        const R cg_ij = (i < D && j < D) ? cgu[i][j] : R(0.0), cg_ji = (i < D && j < D) ? cgu[j][i] : R(0.0);
        R Fsg = R(0.0);
        if (!fj0) Fsg = cg_ij / R(2.) + cg_ji / R(2.) + fu[i] * fu[j] * expn * k13;
        const R Fdl = pi[i + 1][j + 1] * expn;
        R Fdo2, Fds2;
        if (e3) {
          const R common = ch * (t * f2 * (cmd[i + 1] * hy[j + 1][0] * di + cmd[j + 1] * hy[i + 1][0] * dj) +
                                g * (cmd[i + 1] * hy[j + 1][3] * di + cmd[j + 1] * hy[i + 1][3] * dj) * it +
                                f2 * f2 * t * (fu[i] * hy[j + 1][0] + fu[j] * hy[i + 1][0]) +
                                R(2.) * g * f2 * (fu[i] * hy[j + 1][3] + fu[j] * hy[i + 1][3]) * it);
          const R cross = ch * (g * (pi[3][i + 1] * dj + pi[3][j + 1] * di) * it + f2 * (pi[0][i + 1] * dj + pi[0][j + 1] * di) * it);
          Fdo2 = -(-gugjs + sigu - vsig) / R(4.) + (-fu[i] * g * hy[j + 1][0] - fu[j] * g * hy[i + 1][0]) * geo / R(4.) +
                 (common - cross) / R(4.);
          Fds2 = -(-gugjs - sigu + vsig - R(4.) * (fu[i] * fu[j]) * sgu_s * k13) / R(4.) +
                 (-fu[i] * g * hy[j + 1][0] - fu[j] * g * hy[i + 1][0] + R(4.) * fu[i] * fu[j] * hy[0][0] * k13) * geo / R(4.) +
                 (common + cross + ch * (R(4.) * fu[i] * fu[j] * (hy[3][0] * f2 * t + g * hy[3][3] * it + f2 * hy[0][3] * it) * k13)) / R(4.) -
                 pi[i + 1][j + 1] * (g * itc + geo + g * divV) * k13;
        } else {
          Fdo2 = -(-gugjs + sigu - vsig) / R(4.);
          if (fj0) Fds2 = -(-gugjs - sigu + vsig) / R(4.);
          else Fds2 = -(-gugjs - sigu + vsig - R(4.) * (fu[i] * fu[j]) * sgu_s * k13) / R(4.) +
                      (ch * (R(4.) * fu[i] * fu[j] * (g * hy[3][3] * it) * k13)) / R(4.);
          Fds2 = Fds2 - pi[i + 1][j + 1] * (g * itc + g * divV) * k13;
        }
        if (j == 2 && !cart) {
          if (e3) {
            FD2 += g * pi[3][i + 1] * it + f2 * pi[0][i + 1] * it;
            Fsg += -fu[i] * f2 * f2 * t / R(2.) - fu[i] * f2 * g * it;
          } else {
            FD2 += g * pi[3][i + 1] * it;
          }
        }
        if (i == j) {
          Fsg += -cmd[i + 1] * expn * k13;
          if (e3) Fds2 += -cmd[i + 1] * sgu_s * k13 - cmd[i + 1] * hy[0][0] * geo * k13 -
                          ch * (cmd[i + 1] * (hy[3][0] * f2 * t + g * hy[3][3] * it + f2 * hy[0][3] * it) * k13);
          else Fds2 += -cmd[i + 1] * sgu_s * k13 - ch * (cmd[i + 1] * (g * hy[3][3] * it) * k13);
        }
        if (diag) sigF[slot] = Fsg;
        R F = -pi[i + 1][j + 1] - tdelta * Fdl;
        if (e3 || j == 2) F = F - tpi * FD2;   // FD2 vanishes in 2-D off the eta row
        F = F + R(2.) * tpi * Fdo2 * uv - tpp * Fds2;
        if (!fj0) F = F + (R(2.) * eta + lpP * Pi) * Fsg;
        F = (F + phi7 * (fj0 ? sml : sml + fu[i] * fu[j] * ss * k13)) * istg;
        if (i == j) F += phi7 * (-cmd[i + 1] * ss) * (k13 * istg);
        Fext[slot] = F;
#pragma unroll
        for (int kk = 0; kk < D; kk++) {
          R MD2, Msg = R(0.0), Mdo2, Mds2;
          const R Mdl = -pi[i + 1][j + 1] * fuc[kk] * ig;
          if (!fj0) {
            MD2 = g * (fu[i] * hy[j + 1][kk + 1] - fu[i] * hy[j + 1][0] * fuc[kk] * ig + fu[j] * hy[i + 1][kk + 1] -
                       fu[j] * hy[i + 1][0] * fuc[kk] * ig);
            Msg = -fu[i] * fu[j] * fuc[kk] * (k13 * ig);
            Mdo2 = (-fu[i] * hy[j + 1][kk + 1] * g - fu[j] * hy[i + 1][kk + 1] * g + fuc[kk] * fu[i] * hy[j + 1][0] +
                    fuc[kk] * fu[j] * hy[i + 1][0]) / R(4.);
            Mds2 = (-fu[i] * hy[j + 1][kk + 1] * g - fu[j] * hy[i + 1][kk + 1] * g + fuc[kk] * fu[i] * hy[j + 1][0] +
                    fuc[kk] * fu[j] * hy[i + 1][0] + R(4.) * fu[i] * fu[j] * (hy[0][kk + 1] - hy[0][0] * fuc[kk] * ig) * k13 +
                    R(4.) * pi[i + 1][j + 1] * fuc[kk] * k13 * ig) / R(4.);
          } else {
            MD2 = g * (fu[i] * hy[j + 1][kk + 1] - fu[i] * hy[j + 1][0] * fuc[kk] * ig);
            Mdo2 = (-fu[i] * hy[j + 1][kk + 1] * g + fuc[kk] * fu[i] * hy[j + 1][0]) / R(4.);
            Mds2 = (-fu[i] * hy[j + 1][kk + 1] * g + fuc[kk] * fu[i] * hy[j + 1][0] +
                    R(4.) * pi[i + 1][j + 1] * fuc[kk] * k13 * ig) / R(4.);
          }
          if (kk == i) {            // i = k terms
            Mds2 += pi[0][j + 1] / R(4.);
            Mdo2 += -pi[0][j + 1] / R(4.);
            if (!fj0) Msg += -g * fu[j] / R(2.);
          }
          if (kk == j && j < D) {   // j = k terms
            Msg += -g * fu[i] / R(2.);
            Mds2 += pi[0][i + 1] / R(4.);
            Mdo2 += -pi[0][i + 1] / R(4.);
          }
          if (i == j) {             // i = j terms
            Msg += cmd[i + 1] * fuc[kk] * (ig * k13);
            Mds2 += -cmd[i + 1] * (hy[0][kk + 1] - hy[0][0] * fuc[kk] * ig) * k13;
          }
          if (diag) sigM[slot][kk] = Msg;
          R mx = -tpi * MD2 - tdelta * Mdl + R(2.) * tpi * Mdo2 * uv - tpp * Mds2;
          if (!fj0) mx = mx + (R(2.) * eta + lpP * Pi) * Msg;
          Mext[slot][kk] = mx * istg;
        }
      }
    }
  }

  // ---- auxiliary bulk and entropy MRFs (reference :229-362) ---------------
  const R ztil = k.zeta + (k.delta_PiPi - k.tau_Pi) * Pi;
  const R isgT = R(1.0) / (sig * g * T), isgP = R(1.0) / (sig * g * k.tau_Pi);
  R Mb[3], Ms[3];
#pragma unroll
  for (int i = 0; i < D; i++) {
    Mb[i] = (ztil * uc[i] * ig) * isgP;
    Ms[i] = (Pi * uc[i] * ig) * isgT;
  }
  R Fb = -(ztil * expn + Pi) * isgP;
  R Fs = (-Pi * expn) * isgT;
  if (cfg.using_shear) {
    Fs += Fnab * isgT;
    Fb += -(k.lambda_Pipi * Fnab) * isgP;
#pragma unroll
    for (int i = 0; i < D; i++) {
      Mb[i] += -k.lambda_Pipi * Mnab[i] * isgP;
      Ms[i] += Mnab[i] * isgT;
    }
  }
  // ---- four-acceleration (reference :456-618); dN/dt = 0 without diffusion --
  R gP[3], gB[3];
#pragma unroll
  for (int i = 0; i < D; i++) {
    const R f = (D == 2 || i < D - 1) ? -R(1.0) : -R(1.0) * it2;   // make_contravariant
    gP[i] = in.gradP[i] * f;
    gB[i] = in.gradBulk[i] * f;
  }
  const R X = sden * dwds * ig + (rho[0] * dwdr[0] + rho[1] * dwdr[1] + rho[2] * dwdr[2]) * ig;
  R Mw[3];
#pragma unroll
  for (int i = 0; i < D; i++) Mw[i] = X * uc[i] * ig + sig * dwds * Ms[i];
  const R Fw = -X * (e3 ? geo + g * itc + g * divV : g * itc + g * divV) + sig * dwds * Fs;
  const R Fbulk = sig * Fb - Pi * (e3 ? g * divV + g * itc + geo : g * divV + g * itc) * ig;
  R Mu[9], Fu[3];
#pragma unroll
  for (int i = 0; i < D; i++) {
#pragma unroll
    for (int j = 0; j < D; j++) Mu[i * D + j] = u[i] * g * (Mb[j] + Mw[j]) - u[i] * uc[j] * (w + Pi) * ig + M0i[i * D + j];
    Mu[i * D + i] += g * (w + Pi);
    Fu[i] = (gP[i] + gB[i]) - g * (Fw + Fbulk) * u[i] - (w + Pi) * expn * u[i];
    if (e3) Fu[i] = Fu[i] - R(2.) * (w + Pi) * g * uD * dEta(i) * it;
    if (cfg.using_shear) {
      if (e3) Fu[i] += -P(i + 1, 0) * itc - R(2.) * dEta(i) * P(0, 3) * it - in.divshear[i] + in.gradshear[i] - F0i[i];
      else Fu[i] += -P(i + 1, 0) * itc - in.divshear[i] + in.gradshear[i] - F0i[i];
    }
  }
  // ---- diffusion sector: time components of the q MRFs and the charge
  // MRFs, coupled into the four-acceleration -----------------------------------
  R RI[9], MN[3][3], FN[3];
  {   // FP64 form: R = double; mixed form: R = float
    if (dif) {
      const R sig_ = sig, g_ = g;
      // reciprocals once (an FP64 division is a long sequence on the FP64
      // pipe): 1/gamma, 1/t and 1/T
      const R ig_ = ig, it_ = it, iT = R(1.0) / T;
      const R mu[3] = {narrow<R>(th[T_MUB]), narrow<R>(th[T_MUS]), narrow<R>(th[T_MUQ])};
      R RS[3], MS[3] = {0, 0, 0};
      for (int c = 0; c < 3; c++) RS[c] = -mu[c] * iT;
      for (int i = 0; i < D; i++) MS[i] = Ms[i];
      R itq[9], itt[9], itk[9], tqr[9];
      for (int k2 = 0; k2 < 9; k2++) tqr[k2] = narrow<R>(dif->tq[k2]);
      inverse3<R>(tqr, itq);
      for (int c = 0; c < 3; c++)
        for (int d = 0; d < 3; d++) {
          R a1 = R(0.0), a2 = R(0.0);
          for (int kk = 0; kk < 3; kk++) {
            a1 += itq[3 * c + kk] * narrow<R>(dif->tq[3 * kk + d]);
            a2 += itq[3 * c + kk] * narrow<R>(dif->kq[3 * kk + d]);
          }
          itt[3 * c + d] = a1;
          itk[3 * c + d] = a2;
        }
      // Cartesian twin (src/eom_cartesian.cpp:1327-1722): no F_D terms, the
      // expansion rate gamma div v alone, metric without tau
      const R X_ = cart ? g_ * divV : g_ * divV + geo + g_ * it_;
      const R omg = R(1.) - g_ * g_;
      R qc[3][4];
      for (int c = 0; c < 3; c++) {
        qc[c][0] = narrow<R>(dif->q[4 * c]);
        qc[c][1] = -narrow<R>(dif->q[4 * c + 1]);
        qc[c][2] = -narrow<R>(dif->q[4 * c + 2]);
        qc[c][3] = -t2 * narrow<R>(dif->q[4 * c + 3]);
      }
      R F0D[3], F0a[3], A0a[3], R0a[3][3], M0a[3][3], M0D[3][3];
      for (int c = 0; c < 3; c++) {
        const R q0 = narrow<R>(dif->q[4 * c]);
        F0D[c] = cart ? R(0.0)
                      : g_ * g_ * geo * q0 + R(2.) * g_ * g_ * qc[c][3] * u[2] * it_ + t * g_ * qc[c][0] * u[2] * u[2] +
                            t * u[2] * narrow<R>(dif->q[4 * c + 3]);
        F0a[c] = omg * sig_ * narrow<R>(dif->da[c]) * Fs;
        A0a[c] = -omg * narrow<R>(dif->da[c]) * sden * ig_;
        for (int i = 0; i < D; i++) {
          M0D[c][i] = g_ * g_ * (qc[c][i + 1] - qc[c][0] * uc[i] * ig_);
          M0a[c][i] = omg * sig_ * narrow<R>(dif->da[c]) * MS[i];
          F0a[c] += -narrow<R>(dif->ga[3 * i + c]) * u[i] * ig_;
        }
        for (int d = 0; d < 3; d++) {
          R0a[c][d] = omg * sig_ * (narrow<R>(dif->da[c]) * RS[d] + narrow<R>(dif->da[3 + 3 * c + d]));
          A0a[c] += -omg * narrow<R>(dif->da[3 + 3 * c + d]) * rho[d] * ig_;
        }
      }
      // charge MRFs: R_N = gamma sigma 1 - R_0q, M_N = -M_0q, F_N = -F_0q +
      // grad q - div q - q^0 / t (no external sources)
      R RN[9];
      for (int c = 0; c < 9; c++) RN[c] = R(0.0);
      for (int c = 0; c < 3; c++) RN[4 * c] += g_ * sig_;
      for (int c = 0; c < 3; c++) {
        R F0q = R(0.0);
        for (int d = 0; d < 3; d++)
          F0q += (-itt[3 * c + d] * F0D[d] - itq[3 * c + d] * narrow<R>(dif->q[4 * d]) + itk[3 * c + d] * F0a[d] +
                  itk[3 * c + d] * A0a[d] * X_) * ig_ -
                 itt[3 * c + d] * narrow<R>(dif->q[4 * d]) * X_ * ig_;
        for (int i = 0; i < 3; i++) MN[i][c] = R(0.0);
        for (int i = 0; i < D; i++) {
          R acc = R(0.0);
          for (int d = 0; d < 3; d++)
            acc += (-itt[3 * c + d] * M0D[d][i] + itk[3 * c + d] * M0a[d][i] - itk[3 * c + d] * A0a[d] * uc[i] * ig_) *
                       ig_ +
                   itt[3 * c + d] * narrow<R>(dif->q[4 * d]) * uc[i] * ig_ * ig_;
          MN[i][c] = R(0.0) + -acc;
        }
        for (int d = 0; d < 3; d++) {
          R acc = R(0.0);
          for (int kk = 0; kk < 3; kk++) acc += itk[3 * c + kk] * R0a[kk][d] * ig_;
          RN[3 * c + d] += -acc;
        }
        FN[c] = R(0.0);
        if (cart) FN[c] += -F0q + narrow<R>(dif->gq[c]) - narrow<R>(dif->dq[c]);
        else FN[c] += -F0q + narrow<R>(dif->gq[c]) - narrow<R>(dif->dq[c]) - narrow<R>(dif->q[4 * c]) * it_;
      }
      inverse3(RN, RI);
      // R_u = -u gamma (R_w + R_bulk sigma), R_w = sigma dw/drho + sigma dw/ds R_S
      R Ru[3][3];
      for (int i = 0; i < D; i++)
        for (int c = 0; c < 3; c++) {
          const R Rw = sig_ * dwdr[c] + sig_ * dwds * RS[c];
          Ru[i][c] = -u[i] * g_ * (Rw + R(0.0) * sig_);
        }
      for (int i = 0; i < D; i++) {
        R FR = R(0.0);
        for (int j = 0; j < D; j++) {
          R MR = R(0.0);
          for (int c = 0; c < 3; c++)
            for (int d = 0; d < 3; d++) MR += Ru[i][c] * RI[3 * c + d] * MN[j][d];
          Mu[i * D + j] = Mu[i * D + j] - MR;
        }
        for (int c = 0; c < 3; c++)
          for (int d = 0; d < 3; d++) FR += Ru[i][c] * RI[3 * c + d] * FN[d];
        Fu[i] = Fu[i] + FR;
      }
    }
  }
  // du/dt = M^-1 F by cofactors (include/milne.hpp:788-834)
  R du[3];
  if (D == 2) {
    const R idet = R(1.0) / (Mu[0] * Mu[3] - Mu[1] * Mu[2]);
    du[0] = (Mu[3] * idet) * Fu[0] + (-Mu[1] * idet) * Fu[1];
    du[1] = (-Mu[2] * idet) * Fu[0] + (Mu[0] * idet) * Fu[1];
    du[2] = R(0.0);
  } else {
#define A(i, j) Mu[(i) * 3 + (j)]
    const R det = A(0, 0) * A(1, 1) * A(2, 2) + A(0, 1) * A(1, 2) * A(2, 0) + A(0, 2) * A(1, 0) * A(2, 1) -
                       A(0, 2) * A(1, 1) * A(2, 0) - A(0, 1) * A(1, 0) * A(2, 2) - A(0, 0) * A(1, 2) * A(2, 1);
    const R idet = R(1.0) / det;
    const R inv[9] = {(A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) * idet, (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) * idet,
                           (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) * idet, (A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2)) * idet,
                           (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) * idet, (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) * idet,
                           (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0)) * idet, (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) * idet,
                           (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) * idet};
#undef A
#pragma unroll
    for (int i = 0; i < 3; i++) du[i] = inv[i * 3 + 0] * Fu[0] + inv[i * 3 + 1] * Fu[1] + inv[i * 3 + 2] * Fu[2];
  }
  // ---- derivatives (reference :622-826) -------------------------------------
  R m1 = 0, m2 = 0;
#pragma unroll
  for (int i = 0; i < D; i++) { m1 += Ms[i] * du[i]; m2 += Mb[i] * du[i]; o.du[i] = du[i]; }
  o.dS = m1 + Fs;
  o.dBulk = m2 + Fb;
  {   // FP64 form: R = double; mixed form: R = float
    if (dif) {
      // dN/dt = R_N^-1 (F_N + M_N du/dt); the entropy picks up R_S dN/dt;
      // d(ext q)/dt = F_q + M_q du/dt + R_q dN/dt over all three directions
      R MU[3], dN[3];
      for (int c = 0; c < 3; c++) {
        MU[c] = R(0.);
        for (int i = 0; i < D; i++) MU[c] += MN[i][c] * du[i];
      }
      for (int c = 0; c < 3; c++) {
        dN[c] = R(0.);
        for (int d = 0; d < 3; d++) dN[c] += RI[3 * c + d] * (FN[d] + MU[d]);
        dout->dN[c] = widen<R>(dN[c]);
      }
      const R mu[3] = {narrow<R>(th[T_MUB]), narrow<R>(th[T_MUS]), narrow<R>(th[T_MUQ])};
      R RS[3], MS[3] = {0, 0, 0};
      const R iT = R(1.0) / T;
      for (int c = 0; c < 3; c++) RS[c] = -mu[c] * iT;
      for (int i = 0; i < D; i++) MS[i] = Ms[i];
      R rdn = R(0.0);
      for (int c = 0; c < 3; c++) rdn += RS[c] * dN[c];
      o.dS = m1 + Fs + rdn;
      R itq[9], itt[9], itk[9], tqr[9];
      for (int k2 = 0; k2 < 9; k2++) tqr[k2] = narrow<R>(dif->tq[k2]);
      inverse3<R>(tqr, itq);
      for (int c = 0; c < 3; c++)
        for (int d = 0; d < 3; d++) {
          R a1 = R(0.0), a2 = R(0.0);
          for (int kk = 0; kk < 3; kk++) {
            a1 += itq[3 * c + kk] * narrow<R>(dif->tq[3 * kk + d]);
            a2 += itq[3 * c + kk] * narrow<R>(dif->kq[3 * kk + d]);
          }
          itt[3 * c + d] = a1;
          itk[3 * c + d] = a2;
        }
      const R X_ = cart ? g * divV : g * divV + geo + g * it;
      const R gs = g * sig, igs = R(1.0) / gs;
      const R cmd[4] = {R(1.), -R(1.), -R(1.), cart ? -R(1.) : -it * it};
      const R fuc[3] = {-u[0], -u[1], -t2 * u[2]};
      R qc[3][4];
      for (int c = 0; c < 3; c++) {
        qc[c][0] = narrow<R>(dif->q[4 * c]);
        qc[c][1] = -narrow<R>(dif->q[4 * c + 1]);
        qc[c][2] = -narrow<R>(dif->q[4 * c + 2]);
        qc[c][3] = -t2 * narrow<R>(dif->q[4 * c + 3]);
      }
      for (int i = 0; i < 3; i++) {
        const R fui = u[i];
        const R gai[3] = {i < D ? narrow<R>(dif->ga[3 * i]) : R(0.0), i < D ? narrow<R>(dif->ga[3 * i + 1]) : R(0.0),
                               i < D ? narrow<R>(dif->ga[3 * i + 2]) : R(0.0)};
        R FD[3], Fa[3], Aa[3], MD[3][3], Ma[3][3], Ra[3][3];
        for (int c = 0; c < 3; c++) {
          FD[c] = cart ? R(0.0) : fui * g * narrow<R>(dif->q[4 * c]) * geo + R(2.) * fui * qc[c][3] * u[2] * g * it;
          Fa[c] = -fui * g * sig * narrow<R>(dif->da[c]) * Fs + cmd[i + 1] * gai[c];
          Aa[c] = fui * narrow<R>(dif->da[c]) * sden;
          for (int j = 0; j < 3; j++) {
            MD[c][j] = fui * g * (qc[c][j + 1] - qc[c][0] * fuc[j] * ig);
            Ma[c][j] = -fui * g * sig * narrow<R>(dif->da[c]) * MS[j];
          }
          for (int d = 0; d < 3; d++) {
            Ra[c][d] = -fui * g * sig * (narrow<R>(dif->da[c]) * RS[d] + narrow<R>(dif->da[3 + 3 * c + d]));
            Aa[c] += fui * narrow<R>(dif->da[3 + 3 * c + d]) * rho[d];
          }
        }
        for (int c = 0; c < 3; c++) {
          R F = R(0.0), Rq[3];
          for (int d = 0; d < 3; d++) {
            F += (-itt[3 * c + d] * FD[d] - itq[3 * c + d] * narrow<R>(dif->q[4 * d + i + 1]) + itk[3 * c + d] * Fa[d] +
                  itk[3 * c + d] * Aa[d] * X_) * igs;
            R R_ = R(0.0);
            for (int kk = 0; kk < 3; kk++) R_ += itk[3 * c + kk] * Ra[kk][d] * igs;
            Rq[d] = R_;
          }
          R v = F;
          for (int j = 0; j < D; j++) {
            R M = R(0.0);
            for (int d = 0; d < 3; d++)
              M += (-itt[3 * c + d] * MD[d][j] + itk[3 * c + d] * Ma[d][j] - itk[3 * c + d] * Aa[d] * fuc[j] * ig) * igs;
            v += M * du[j];
          }
          for (int d = 0; d < 3; d++) v += Rq[d] * dN[d];
          dout->dQ[3 * c + i] = widen<R>(v);
        }
      }
    }
  }
#pragma unroll
  for (int sl = 0; sl < 5; sl++) {
    R acc = R(0.0);
#pragma unroll
    for (int kk = 0; kk < D; kk++) acc += Mext[sl][kk] * du[kk];
    o.dShv[sl] = cfg.using_shear ? acc + Fext[sl] : R(0.0);
  }
  if (diag) {
    R c1 = R(0.0);
#pragma unroll
    for (int i = 0; i < D; i++) c1 += uc[i] * du[i];
    diag[0] = -R(1.) * c1 / g + g * divV + (cart ? R(0.0) : g / t) + geo;
#pragma unroll
    for (int sl = 0; sl < 5; sl++) {
      R acc = R(0.0);
#pragma unroll
      for (int kk = 0; kk < D; kk++) acc += sigM[sl][kk] * du[kk];
      diag[1 + sl] = acc + sigF[sl];
    }
    R m3 = R(0.0);
#pragma unroll
    for (int i = 0; i < D; i++) m3 += Mnab[i] * du[i];
    diag[6] = m3 + Fnab;
  }
  // ---- dEz (reference :827-862) ---------------------------------------------
  const R u3 = (D == 3) ? u[2] : R(0.0);
  o.dEz = ((narrow<R>(th[T_E]) + narrow<R>(th[T_P]) + Pi) * u3 * u3 + (narrow<R>(th[T_P]) + Pi) * it2 + P(3, 3)) * in.m * t2 /
          in.sigma_lab;
}

}  // namespace ccake
