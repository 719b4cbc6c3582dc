// CPU oracle: analytic equations of state, the (e|s, B, S, Q) -> (T, mu) root
// finder with the reference's seed chain, and the derived thermodynamics.
// TEST INFRASTRUCTURE ONLY (see oracle.hpp).
#include "oracle.hpp"
#include "table_oracle.hpp"

#include <algorithm>
#include <cmath>

namespace orc {

namespace {

struct Scales { double c, T0, muB0, muQ0, muS0; };

// Reference EoS chains (src/eos_initialization.cpp:216-501):
//   conformal           -> [conformal, conformal_diagonal]
//   conformal_diagonal  -> [conformal_diagonal]
//   table               -> [table, tanh_conformal, conformal, conformal_diagonal]
//                          (use_tanh_conformal = true, include/eos_header.h:7)
enum Model { mConformal = 0, mConfDiag = 1, mTable = 2, mTanh = 3 };

int chain_model(const Config& c, int k) {
  if (c.eos_kind == kConformal) return k == 0 ? mConformal : mConfDiag;
  if (c.eos_kind == kConformalDiagonal) return mConfDiag;
  return k == 0 ? mTable : (k == 1 ? mTanh : (k == 2 ? mConformal : mConfDiag));
}

// The tanh-conformal fallback is matched to the table by the same rule as the
// conformal one (src/eos_initialization.cpp:276-341, :343-403): same scales.
Scales model_scales(const Config& c, const Table* tab, int model) {
  if (c.eos_kind == kTable && tab && model != mTable) {
    const auto& k = model == mConfDiag ? tab->cdiag : tab->conf;
    return {k.c, k.T0, k.muB0, k.muQ0, k.muS0};
  }
  return {c.eos_c, c.eos_T0, c.eos_muB0, c.eos_muQ0, c.eos_muS0};
}

// include/eos_conformal.h:33-194: p = c T0^4 x^2, x = (T/T0)^2 + sum (mu/mu0)^2.
void conformal_thermo(const Scales& k, const double* x4, double* o) {
  const double T = x4[0], mB = x4[1], mQ = x4[2], mS = x4[3];
  const double x = (T / k.T0) * (T / k.T0) + (mB / k.muB0) * (mB / k.muB0) +
                   (mS / k.muS0) * (mS / k.muS0) + (mQ / k.muQ0) * (mQ / k.muQ0);
  const double cp = k.c * k.T0 * k.T0 * k.T0 * k.T0;
  const double p = cp * x * x;
  const double s = 4.0 * cp * T * x / (k.T0 * k.T0);
  const double B = 4.0 * cp * mB * x / (k.muB0 * k.muB0);
  const double S = 4.0 * cp * mS * x / (k.muS0 * k.muS0);
  const double Q = 4.0 * cp * mQ * x / (k.muQ0 * k.muQ0);
  o[0] = p; o[1] = s; o[2] = B; o[3] = S; o[4] = Q;
  o[5] = (s * T + mB * B + mQ * Q + mS * S) - p;
  o[6] = 1.0 / 3.0;
  o[7] = cp * (8.0 * mB * mB / (k.muB0 * k.muB0 * k.muB0 * k.muB0) + 4.0 * x / (k.muB0 * k.muB0));
  o[8] = cp * (8.0 * mQ * mQ / (k.muQ0 * k.muQ0 * k.muQ0 * k.muQ0) + 4.0 * x / (k.muQ0 * k.muQ0));
  o[9] = cp * (8.0 * mS * mS / (k.muS0 * k.muS0 * k.muS0 * k.muS0) + 4.0 * x / (k.muS0 * k.muS0));
  o[10] = 8.0 * cp * mB * mQ / (k.muB0 * k.muB0 * k.muQ0 * k.muQ0);
  o[11] = 8.0 * cp * mB * mS / (k.muB0 * k.muB0 * k.muS0 * k.muS0);
  o[12] = 8.0 * cp * mS * mQ / (k.muS0 * k.muS0 * k.muQ0 * k.muQ0);
  o[13] = 8.0 * cp * T * mB / (k.T0 * k.T0 * k.muB0 * k.muB0);
  o[14] = 8.0 * cp * T * mQ / (k.T0 * k.T0 * k.muQ0 * k.muQ0);
  o[15] = 8.0 * cp * T * mS / (k.T0 * k.T0 * k.muS0 * k.muS0);
  o[16] = cp * (8.0 * T * T / (k.T0 * k.T0 * k.T0 * k.T0) + 4.0 * x / (k.T0 * k.T0));
}

// include/eos_conformal_diagonal.h:78-205: p = c T0^4 [(T/T0)^4 + sum (mu/mu0)^4];
// the cross susceptibilities are the placeholder TINY, as in the reference.
void confdiag_thermo(const Scales& k, const double* x4, double* o) {
  const double T = x4[0], mB = x4[1], mQ = x4[2], mS = x4[3];
  const double cp = k.c * k.T0 * k.T0 * k.T0 * k.T0;
  auto q4 = [](double a, double b) { double r = a / b; return r * r * r * r; };
  const double p = cp * (q4(T, k.T0) + q4(mB, k.muB0) + q4(mS, k.muS0) + q4(mQ, k.muQ0));
  const double s = 4.0 * cp * T * T * T / (k.T0 * k.T0 * k.T0 * k.T0);
  const double B = 4.0 * cp * mB * mB * mB / (k.muB0 * k.muB0 * k.muB0 * k.muB0);
  const double S = 4.0 * cp * mS * mS * mS / (k.muS0 * k.muS0 * k.muS0 * k.muS0);
  const double Q = 4.0 * cp * mQ * mQ * mQ / (k.muQ0 * k.muQ0 * k.muQ0 * k.muQ0);
  o[0] = p; o[1] = s; o[2] = B; o[3] = S; o[4] = Q;
  o[5] = (s * T + mB * B + mQ * Q + mS * S) - p;
  o[6] = 1.0 / 3.0;
  o[7] = 12.0 * cp * mB * mB / (k.muB0 * k.muB0 * k.muB0 * k.muB0);
  o[8] = 12.0 * cp * mQ * mQ / (k.muQ0 * k.muQ0 * k.muQ0 * k.muQ0);
  o[9] = 12.0 * cp * mS * mS / (k.muS0 * k.muS0 * k.muS0 * k.muS0);
  for (int i = 10; i < 16; i++) o[i] = kTiny;
  o[16] = 12.0 * cp * T * T / (k.T0 * k.T0 * k.T0 * k.T0);
}

void solve4(double A[4][4], double* b, double* xout);

// include/eos_tanh_conformal.h: p = t(T) p_conformal with
// t = (1 + tanh((T - Tc)/Ts))/2, Tc = 220 MeV, Ts = 120 MeV
// (src/eos_initialization.cpp:334-335); derivatives by the product rule.
// c_s^2: the adiabatic speed of sound (dp/de at fixed s : rho ratios),
// n . chi^-1 . n / (T s + mu . rho) with n = grad p and chi its Hessian.
void tanh_conformal_thermo(const Scales& k, const double* x4, double* o) {
  const double Tc = 220.0 / kHbarcMeVfm, Ts = 120.0 / kHbarcMeVfm;
  double pc[17];
  conformal_thermo(k, x4, pc);
  const double T = x4[0], mB = x4[1], mQ = x4[2], mS = x4[3];
  const double arg = (T - Tc) / Ts;
  const double tanh_a = std::tanh(arg), sech_a = 1.0 / std::cosh(arg);
  const double f = 0.5 * (1.0 + tanh_a);
  const double f1 = 0.5 * sech_a * sech_a / Ts;
  const double f2 = -2.0 * tanh_a * f1 / Ts;
  o[0] = f * pc[0];
  o[1] = f * pc[1] + f1 * pc[0];
  o[2] = f * pc[2];
  o[3] = f * pc[3];
  o[4] = f * pc[4];
  o[5] = (o[1] * T + mB * o[2] + mQ * o[4] + mS * o[3]) - o[0];
  for (int i = 7; i <= 12; i++) o[i] = f * pc[i];
  o[13] = f * pc[13] + f1 * pc[2];   // chi_TB
  o[14] = f * pc[14] + f1 * pc[4];   // chi_TQ
  o[15] = f * pc[15] + f1 * pc[3];   // chi_TS
  o[16] = f * pc[16] + 2.0 * f1 * pc[1] + f2 * pc[0];
  double chi[4][4] = {{o[16], o[13], o[14], o[15]},
                      {o[13], o[7], o[10], o[11]},
                      {o[14], o[10], o[8], o[12]},
                      {o[15], o[11], o[12], o[9]}};
  double grad[4] = {o[1], o[2], o[4], o[3]}, rhs[4] = {o[1], o[2], o[4], o[3]}, sol[4];
  solve4(chi, rhs, sol);
  double q = 0.0;
  for (int i = 0; i < 4; i++) q += grad[i] * sol[i];
  o[6] = q / (o[1] * T + mB * o[2] + mQ * o[4] + mS * o[3]);
}

void model_thermo(const Config& c, const Table* tab, int model, const double* x4, double* o) {
  if (model == mTable) { table_full_thermo(*tab, x4, o); return; }
  Scales k = model_scales(c, tab, model);
  if (model == mConformal) conformal_thermo(k, x4, o);
  else if (model == mTanh) tanh_conformal_thermo(k, x4, o);
  else confdiag_thermo(k, x4, o);
}

// Densities (e|s, B, Q, S) and their Jacobian with respect to (T, muB, muQ, muS).
// The reference's GSL hybrid solver differentiates the density function
// numerically; here the exact derivative of the same function is used. For the
// conformal-diagonal model that Jacobian is diagonal (its tabulated TINY cross
// terms are placeholders, not derivatives).
// For the table the Jacobian is that of the interpolated densities (the
// function the solver zeroes; the reference's GSL hybrids solver
// differentiates it by finite differences), not the interpolated
// susceptibilities.
// Reduced modes of the reference for a model whose chemical-potential axes
// are frozen (a table with one node along them). Derivatives
// (src/eos.cpp:129-141): 2 every mu frozen (T-only), 1 muQ and muS frozen
// (baryon-only), else 0. Root finder (src/rootfinder.cpp:447-491): the same,
// and only with zero target charges (T-only: B, Q, S; baryon-only: Q, S).
int frozen_mode(const Table* tab, int model) {
  if (model != mTable || !tab) return 0;
  const bool fb = tab->n[1] <= 1, fq = tab->n[2] <= 1, fs = tab->n[3] <= 1;
  if (fb && fq && fs) return 2;
  return (fq && fs) ? 1 : 0;
}
int root_mode(const Table* tab, int model, const double* tgt) {   // tgt order (e|s, B, Q, S)
  if (model != mTable || !tab) return 0;
  const bool fb = tab->n[1] <= 1, fq = tab->n[2] <= 1, fs = tab->n[3] <= 1;
  const bool zb = std::fabs(tgt[1]) < 1e-30, zq = std::fabs(tgt[2]) < 1e-30, zs = std::fabs(tgt[3]) < 1e-30;
  if (fb && fq && fs && zb && zq && zs) return 2;
  return (fq && fs && zq && zs) ? 1 : 0;
}

void densities_and_jacobian(const Config& c, const Table* tab, int model, int entropy,
                            const double* x, double* f, double J[4][4], int rmode = 0);

// In a reduced mode the equations of the frozen chemical potentials are
// mu = 0 (src/rootfinder.cpp:119-140), with the targets of those charges 0.
void reduce_rows(int rmode, const double* x, double* f, double J[4][4]) {
  for (int i = (rmode == 2 ? 1 : 2); rmode && i < 4; i++) {
    f[i] = x[i];
    for (int j = 0; j < 4; j++) J[i][j] = (i == j) ? 1.0 : 0.0;
  }
}

void densities_and_jacobian(const Config& c, const Table* tab, int model, int entropy,
                            const double* x, double* f, double J[4][4], int rmode) {
  double o[17];
  if (model == mTable) {
    double jac[5][4];
    table_full_thermo(*tab, x, o, jac);
    f[0] = entropy ? o[1] : o[5];
    f[1] = o[2];
    f[2] = o[4];
    f[3] = o[3];
    for (int j = 0; j < 4; j++) {
      J[0][j] = entropy ? jac[0][j] : jac[4][j];
      J[1][j] = jac[1][j];
      J[2][j] = jac[3][j];
      J[3][j] = jac[2][j];
    }
    reduce_rows(rmode, x, f, J);
    return;
  }
  model_thermo(c, tab, model, x, o);
  // Hessian of p in (T, muB, muQ, muS) order
  double H[4][4];
  if (model == mConfDiag) {
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) H[i][j] = 0.0;
    H[0][0] = o[16]; H[1][1] = o[7]; H[2][2] = o[8]; H[3][3] = o[9];
  } else {
    H[0][0] = o[16]; H[0][1] = H[1][0] = o[13]; H[0][2] = H[2][0] = o[14]; H[0][3] = H[3][0] = o[15];
    H[1][1] = o[7]; H[1][2] = H[2][1] = o[10]; H[1][3] = H[3][1] = o[11];
    H[2][2] = o[8]; H[2][3] = H[3][2] = o[12]; H[3][3] = o[9];
  }
  f[0] = entropy ? o[1] : o[5];
  f[1] = o[2];
  f[2] = o[4];
  f[3] = o[3];
  for (int j = 0; j < 4; j++) {
    J[1][j] = H[1][j];
    J[2][j] = H[2][j];
    J[3][j] = H[3][j];
    if (entropy) J[0][j] = H[0][j];
    else J[0][j] = x[0] * H[0][j] + x[1] * H[1][j] + x[2] * H[2][j] + x[3] * H[3][j];
  }
}

// Gaussian elimination with partial pivoting; an exactly-zero pivot column
// (a decoupled unknown) gets a zero step.
void solve4(double A[4][4], double* b, double* xout) {
  int piv[4] = {0, 1, 2, 3};
  bool dead[4] = {false, false, false, false};
  for (int k = 0; k < 4; k++) {
    int p = k;
    double best = std::fabs(A[k][k]);
    for (int i = k + 1; i < 4; i++)
      if (std::fabs(A[i][k]) > best) { best = std::fabs(A[i][k]); p = i; }
    if (p != k) {
      for (int j = 0; j < 4; j++) std::swap(A[k][j], A[p][j]);
      std::swap(b[k], b[p]);
      std::swap(piv[k], piv[p]);
    }
    if (A[k][k] == 0.0) { dead[k] = true; continue; }
    for (int i = k + 1; i < 4; i++) {
      double m = A[i][k] / A[k][k];
      if (m == 0.0) continue;
      for (int j = k; j < 4; j++) A[i][j] -= m * A[k][j];
      b[i] -= m * b[k];
    }
  }
  for (int k = 3; k >= 0; k--) {
    if (dead[k]) { xout[k] = 0.0; continue; }
    double acc = b[k];
    for (int j = k + 1; j < 4; j++) acc -= A[k][j] * xout[j];
    xout[k] = acc / A[k][k];
  }
}

// max(a, b) that returns NaN when either is NaN
inline double nan_max(double a, double b) { return (b > a || b != b) ? b : a; }

// One solver attempt from a seed (replaces GSL hybrids in src/rootfinder.cpp:206-416).
// Stopping rule: the reference's max |F_i| < 1e-10 (gsl_multiroot_test_residual,
// include/rootfinder.h:36-37); once it holds, full Newton steps continue (at
// most 8) until the largest relative step is below 1e-12, so the answer does
// not depend on where the absolute rule happened to trigger. At most 100
// iterations; leaving the model's (T, mu) box fails the attempt.
bool newton_attempt(const Config& c, const Table* tab, int model, int entropy,
                    const double* tgt, const double* lo, const double* hi, double* x, int* iters, int rmode = 0) {
  const double tol = 1e-10;
  int extra = -1, nslow1 = 0, nslow2 = 0;
  double xgood[4] = {0, 0, 0, 0};
  for (int it = 0; it < 100; it++) {
    double f[4], J[4][4];
    densities_and_jacobian(c, tab, model, entropy, x, f, J, rmode);
    double F[4] = {f[0] - tgt[0], f[1] - tgt[1], f[2] - tgt[2], f[3] - tgt[3]};
    // maxima propagate NaN (std::max(a, NaN) would return a): a NaN residual
    // fails the iterate, as GSL_EBADFUNC fails the reference's solver
    double fmax = 0;
    for (int i = 0; i < 4; i++) fmax = nan_max(fmax, std::fabs(F[i]));
    if (!(fmax <= 1e300)) { *iters += it + 1; return false; }  // NaN or infinite
    if (extra < 0 && fmax < tol) extra = 0;
    double rhs[4] = {-F[0], -F[1], -F[2], -F[3]}, dx[4];
    solve4(J, rhs, dx);
    if (extra >= 0) {
      // x met the residual test. Full steps continue (at most 8) until the
      // relative step is below 1e-12; each is verified at the next iteration
      // and, if its residual left the tolerance, the last verified point is
      // returned (the point the reference's solver stops at).
      if (extra > 0 && !(fmax < tol)) {
        for (int i = 0; i < 4; i++) x[i] = xgood[i];
        *iters += it;
        return true;
      }
      double y[4], rel = 0;
      bool inbox = true;
      for (int i = 0; i < 4; i++) {
        xgood[i] = x[i];
        y[i] = x[i] + dx[i];
        rel = std::max(rel, std::fabs(dx[i]) / std::max(std::fabs(x[i]), 1e-300));
        // every iterate stays in the model's box (src/rootfinder.cpp:277-330)
        inbox = inbox && (y[i] >= lo[i] && y[i] <= hi[i]);
      }
      const bool usable = y[0] > 0 && std::isfinite(y[0]) && inbox;
      if (rel < 1e-12) {
        if (usable) for (int i = 0; i < 4; i++) x[i] = y[i];
        *iters += it + 1;
        return true;
      }
      if (extra >= 8 || !usable) { *iters += it + 1; return true; }
      for (int i = 0; i < 4; i++) x[i] = y[i];
      extra++;
      continue;
    }
    // damped step: halve while the residual grows (at most 6 halvings)
    double lam = 1.0;
    double y[4];
    for (int h = 0; h < 7; h++) {
      for (int i = 0; i < 4; i++) y[i] = x[i] + lam * dx[i];
      if (y[0] > 0) {
        double fy[4], Jy[4][4];
        densities_and_jacobian(c, tab, model, entropy, y, fy, Jy, rmode);
        double gmax = 0;
        for (int i = 0; i < 4; i++) gmax = nan_max(gmax, std::fabs(fy[i] - tgt[i]));
        if (gmax <= fmax || h == 6) break;
      }
      lam *= 0.5;
    }
    bool have = y[0] > 0;
    if (!(y[0] > 0)) y[0] = 0.5 * x[0];
    // progress test of the reference's solver (GSL hybrids, called from
    // src/rootfinder.cpp:206-416): the actual relative reduction of |F|^2;
    // five iterations below 0.1 or ten below 0.001 fail the attempt
    if (have) {
      double fy[4], Jy[4][4];
      densities_and_jacobian(c, tab, model, entropy, y, fy, Jy, rmode);
      double n0 = 0.0, n1 = 0.0;
      for (int i = 0; i < 4; i++) {
        n0 += F[i] * F[i];
        const double r = fy[i] - tgt[i];
        n1 += r * r;
      }
      const double actred = n0 > 0.0 ? 1.0 - n1 / n0 : 0.0;
      nslow1 = actred >= 0.001 ? 0 : nslow1 + 1;
      nslow2 = actred >= 0.1 ? 0 : nslow2 + 1;
    } else {
      nslow1++;
      nslow2++;
    }
    for (int i = 0; i < 4; i++) x[i] = y[i];
    for (int i = 0; i < 4; i++)
      if (!(x[i] >= lo[i] && x[i] <= hi[i])) { *iters += it + 1; return false; }
    if (nslow2 >= 5 || nslow1 >= 10) { *iters += it + 1; return false; }
  }
  *iters += 100;
  return false;
}

double sgn(double v) { return (0.0 < v) - (v < 0.0); }

void model_box(const Config& c, const Table* tab, int model, double* lo, double* hi) {
  if (model == mTable) { table_box(*tab, lo, hi); return; }
  lo[0] = 0.0; hi[0] = kTbqsInf;
  for (int i = 1; i < 4; i++) { lo[i] = -kTbqsInf; hi[i] = kTbqsInf; }
}

// src/rootfinder.cpp:421-715 (find_root): seed sanitising and the ladder of
// perturbed restarts (T +-20%, muB +-20%, muS +-20%, muQ +-20%, then signed
// default chemical potentials).
bool find_root(const Config& c, const Table* tab, int model, int entropy, const double* tgt,
               double* x, int* iters) {
  double lo[4], hi[4];
  model_box(c, tab, model, lo, hi);
  const double TOL = 1e-10;
  double pos[4] = {x[0], x[1], x[2], x[3]};
  // the reduced modes start the frozen potentials at zero
  const int rmode = root_mode(tab, model, tgt);
  for (int i = (rmode == 2 ? 1 : 2); rmode && i < 4; i++) pos[i] = 0.0;
  const double sg[4] = {1.0, sgn(tgt[1]), sgn(tgt[2]), sgn(tgt[3])};
  for (int i = 0; i < 4; i++)
    if (pos[i] * pos[i] < TOL) pos[i] = std::min(0.5 * hi[i], 1.0) * sg[i];
  auto attempt = [&](double a, double b, double q, double s_) {
    double y[4] = {a, b, q, s_};
    if (newton_attempt(c, tab, model, entropy, tgt, lo, hi, y, iters, rmode)) {
      for (int i = 0; i < 4; i++) x[i] = y[i];
      return true;
    }
    return false;
  };
  // out-of-range restarts leave the position unchanged (src/rootfinder.cpp:181-210)
  auto clampT = [&](double v) { return (v < lo[0] || v > hi[0]) ? pos[0] : v; };
  const double t0 = pos[0], b0 = pos[1], q0 = pos[2], s0 = pos[3];
  if (attempt(t0, b0, q0, s0)) return true;
  double tp = t0 + 0.2 * t0 > hi[0] ? hi[0] - 1 : t0 + 0.2 * t0;
  if (attempt(clampT(tp), b0, q0, s0)) return true;
  double tm = t0 - 0.2 * t0 < lo[0] ? lo[0] + 1 : t0 - 0.2 * t0;
  if (attempt(clampT(tm), b0, q0, s0)) return true;
  double bp = b0 + 0.2 * b0 > hi[1] ? hi[1] - 1 : b0 + 0.2 * b0;
  if (attempt(t0, bp, q0, s0)) return true;
  double bm = b0 - 0.2 * b0 < lo[1] ? lo[1] + 1 : b0 - 0.2 * b0;
  if (attempt(t0, bm, q0, s0)) return true;
  double sp = s0 + 0.2 * s0 > hi[3] ? hi[3] - 1 : s0 + 0.2 * s0;
  if (attempt(t0, b0, q0, sp)) return true;
  double sm = s0 - 0.2 * s0 < lo[3] ? lo[3] + 1 : s0 - 0.2 * s0;
  if (attempt(t0, b0, q0, sm)) return true;
  double qp = q0 + 0.2 * q0 > hi[2] ? hi[2] - 1 : q0 + 0.2 * q0;
  if (attempt(t0, b0, qp, s0)) return true;
  double qm = q0 - 0.2 * q0 < lo[2] ? lo[2] + 1 : q0 - 0.2 * q0;
  if (attempt(t0, b0, qm, s0)) return true;
  if (attempt(t0, std::min(0.5 * hi[1], 1.0) * sg[1], std::min(0.5 * hi[2], 1.0) * sg[2],
              std::min(0.5 * hi[3], 1.0) * sg[3]))
    return true;
  return false;
}

// include/eos_conformal_diagonal.h:49-76: exact inverses of the diagonal model,
// used by the reference as the last seed of the chain.
void confdiag_seed(const Scales& k, int entropy, const double* tgt, double* x) {
  const double den = 1.5874010519681994748 * std::pow(k.c, 1.0 / 3.0);
  const double e0 = tgt[0], B = tgt[1], Q = tgt[2], S = tgt[3];
  if (entropy) {
    x[0] = std::pow(k.T0 * k.T0 * k.T0 * k.T0 * e0, 1.0 / 3.0) / den;
  } else {
    const double ft = 4.0 / 3.0;
    double disc = e0 - 3.0 * (std::pow(k.muB0 * std::fabs(B), ft) + std::pow(k.muS0 * std::fabs(S), ft) +
                              std::pow(k.muQ0 * std::fabs(Q), ft)) / (4.0 * den);
    x[0] = k.T0 * std::pow(disc / (3.0 * k.c), 0.25);
  }
  x[1] = sgn(B) * std::pow(k.muB0 * k.muB0 * k.muB0 * k.muB0 * std::fabs(B), 1.0 / 3.0) / den;
  x[2] = sgn(Q) * std::pow(k.muQ0 * k.muQ0 * k.muQ0 * k.muQ0 * std::fabs(Q), 1.0 / 3.0) / den;
  x[3] = sgn(S) * std::pow(k.muS0 * k.muS0 * k.muS0 * k.muS0 * std::fabs(S), 1.0 / 3.0) / den;
}

}  // namespace

int eos_chain_length(const Config& c) {
  return c.eos_kind == kConformal ? 2 : (c.eos_kind == kConformalDiagonal ? 1 : 4);
}

void eos_full_thermo(const Config& c, const Table* tab, int k, const double tbqs[4], double out[17]) {
  model_thermo(c, tab, chain_model(c, k), tbqs, out);
}

// src/eos.cpp:629-804 (rootfinder_update_s, entropy mode) and :813-975
// (rootfinder_s_out, energy mode). Target order (e|s, B, S, Q); result order
// (T, muB, muQ, muS). Returns the chain index used, -1 when no model solved.
int eos_invert(const Config& c, const Table* tab, int entropy, const double target[4],
               int start_model, double x[4], int* iterations) {
  // root-finder target order is (e|s, B, Q, S)
  const double tgt[4] = {target[0], target[1], target[3], target[2]};
  const int n = eos_chain_length(c);
  const Scales cdk = model_scales(c, tab, mConfDiag);
  int it = 0;
  const double prev[4] = {x[0], x[1], x[2], x[3]};
  for (int k = (entropy ? std::max(0, start_model) : 0); k < n; k++) {
    const int model = chain_model(c, k);
    double y[4];
    bool ok;
    if (entropy) {
      // previous location, then zero chemical potentials, then the forced seed,
      // then the conformal-diagonal analytic seed (src/eos.cpp:661-702)
      for (int i = 0; i < 4; i++) y[i] = prev[i];
      ok = find_root(c, tab, model, 1, tgt, y, &it);
      if (!ok) { y[0] = prev[0]; y[1] = y[2] = y[3] = 0.0; ok = find_root(c, tab, model, 1, tgt, y, &it); }
      if (!ok) {
        y[0] = 580.0 / kHbarcMeVfm; y[1] = sgn(tgt[1]); y[2] = sgn(tgt[2]); y[3] = sgn(tgt[3]);
        ok = find_root(c, tab, model, 1, tgt, y, &it);
      }
      if (!ok) { confdiag_seed(cdk, 1, target, y); ok = find_root(c, tab, model, 1, tgt, y, &it); }
    } else {
      // forced seed, then the conformal-diagonal seed (src/eos.cpp:843-870)
      y[0] = 580.0 / kHbarcMeVfm; y[1] = sgn(tgt[1]); y[2] = sgn(tgt[2]); y[3] = sgn(tgt[3]);
      ok = find_root(c, tab, model, 0, tgt, y, &it);
      if (!ok) { confdiag_seed(cdk, 0, target, y); ok = find_root(c, tab, model, 0, tgt, y, &it); }
    }
    // a solution is a finite point with T > 0
    ok = ok && y[0] > 0.0 && y[0] <= 1e300 && std::fabs(y[1]) <= 1e300 && std::fabs(y[2]) <= 1e300 &&
         std::fabs(y[3]) <= 1e300;
    if (ok) {
      double o[17];
      model_thermo(c, tab, model, y, o);
      // prohibit_unstable_cs2 / prohibit_acausal_cs2 default true (include/settings.h:145-147)
      if (!(o[6] >= 0.0 && o[6] <= 1.0)) continue;
      // restrict_mu_T_ratios (src/eos.cpp:781-786): a table solution with a
      // chemical potential above 3.5 T is refused
      if (c.restrict_mu_T_ratios && model == mTable &&
          std::max(std::max(std::fabs(y[1]), std::fabs(y[3])), std::fabs(y[2])) > 3.5 * y[0])
        continue;
      for (int i = 0; i < 4; i++) x[i] = y[i];
      if (iterations) *iterations = it;
      return k;
    }
  }
  if (iterations) *iterations = it;
  return -1;
}

namespace {
// src/eos_derivatives.cpp:457-560 (deriv_mult_aTm_1b): a^T m^-1 b with the
// reference's guard on small diagonal entries m11, m22 (|m| < 1e-3 -> +-1e-3).
double aTmb(const double a[3], double m[3][3], const double b[3]) {
  const double EPS = 1e-3;
  if (std::fabs(m[1][1]) < EPS) m[1][1] = (m[1][1] >= 0.0 ? EPS : -EPS);
  if (std::fabs(m[2][2]) < EPS) m[2][2] = (m[2][2] >= 0.0 ? EPS : -EPS);
  // LU with partial pivoting (the reference uses gsl_linalg_LU_decomp/invert)
  double A[3][3], y[3] = {b[0], b[1], b[2]};
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) A[i][j] = m[i][j];
  for (int k = 0; k < 3; k++) {
    int p = k;
    for (int i = k + 1; i < 3; i++) if (std::fabs(A[i][k]) > std::fabs(A[p][k])) p = i;
    if (p != k) { for (int j = 0; j < 3; j++) std::swap(A[k][j], A[p][j]); std::swap(y[k], y[p]); }
    for (int i = k + 1; i < 3; i++) {
      double f = A[i][k] / A[k][k];
      for (int j = k; j < 3; j++) A[i][j] -= f * A[k][j];
      y[i] -= f * y[k];
    }
  }
  double z[3];
  for (int k = 2; k >= 0; k--) {
    double acc = y[k];
    for (int j = k + 1; j < 3; j++) acc -= A[k][j] * z[j];
    z[k] = acc / A[k][k];
  }
  return a[0] * z[0] + a[1] * z[1] + a[2] * z[2];
}

struct Chi { double t2, tb, tq, ts, b2, q2, s2, bq, bs, sq; };

// The reduced modes of the terms (rm: 2 T-only, 1 baryon-only; src/
// eos_derivatives.cpp:33-45, :74-90, :160-172, :240-254): the Schur
// complements over the active rows only, with the reference's 1e-30 guards.
double term1(const Chi& x, int rm = 0) {
  if (rm == 2) return x.t2;
  if (rm == 1) return x.t2 - (x.tb * x.tb) / (x.b2 + 1e-30);
  double a[3] = {x.tb, x.ts, x.tq};
  double m[3][3] = {{x.b2, x.bs, x.bq}, {x.bs, x.s2, x.sq}, {x.bq, x.sq, x.q2}};
  return x.t2 - aTmb(a, m, a);
}
// :75-155 (calc_term_2), i = 0 B, 1 S, 2 Q
double term2(const Chi& x, int i, int rm = 0) {
  if (rm == 2) return 0.0;
  if (rm == 1) return i == 0 ? x.tb - (x.t2 * x.b2) / (x.tb + 1e-30) : 0.0;
  if (i == 0) {
    double a[3] = {x.t2, x.ts, x.tq}, b[3] = {x.b2, x.bs, x.bq};
    double m[3][3] = {{x.tb, x.bs, x.bq}, {x.ts, x.s2, x.sq}, {x.tq, x.sq, x.q2}};
    return x.tb - aTmb(a, m, b);
  } else if (i == 1) {
    double a[3] = {x.t2, x.tb, x.tq}, b[3] = {x.bs, x.s2, x.sq};
    double m[3][3] = {{x.tb, x.b2, x.bq}, {x.ts, x.bs, x.sq}, {x.tq, x.bq, x.q2}};
    return x.ts - aTmb(a, m, b);
  }
  double a[3] = {x.t2, x.tb, x.ts}, b[3] = {x.bq, x.sq, x.q2};
  double m[3][3] = {{x.tb, x.b2, x.bs}, {x.ts, x.bs, x.s2}, {x.tq, x.bq, x.sq}};
  return x.tq - aTmb(a, m, b);
}
// :157-233 (calc_term_3)
double term3(const Chi& x, int i, int rm = 0) {
  if (rm == 2) return 0.0;
  if (rm == 1) return i == 0 ? x.tb - (x.b2 * x.t2) / (x.tb + 1e-30) : 0.0;
  if (i == 0) {
    double a[3] = {x.b2, x.bs, x.bq}, b[3] = {x.t2, x.ts, x.tq};
    double m[3][3] = {{x.tb, x.ts, x.tq}, {x.bs, x.s2, x.sq}, {x.bq, x.sq, x.q2}};
    return x.tb - aTmb(a, m, b);
  } else if (i == 1) {
    double a[3] = {x.bs, x.s2, x.sq}, b[3] = {x.t2, x.tb, x.tq};
    double m[3][3] = {{x.tb, x.ts, x.tq}, {x.b2, x.bs, x.bq}, {x.bq, x.sq, x.q2}};
    return x.ts - aTmb(a, m, b);
  }
  double a[3] = {x.bq, x.sq, x.q2}, b[3] = {x.t2, x.tb, x.ts};
  double m[3][3] = {{x.tb, x.ts, x.tq}, {x.b2, x.bs, x.bq}, {x.bs, x.s2, x.sq}};
  return x.tq - aTmb(a, m, b);
}
// :235-455 (calc_term_4(j, i)), indices 0 B, 1 S, 2 Q
double term4(const Chi& x, int j, int i, int rm = 0) {
  if (rm == 2) return 0.0;
  if (rm == 1) return (i == 0 && j == 0) ? x.b2 - (x.tb * x.tb) / (x.t2 + 1e-30) : 0.0;
  double a[3], b[3], m[3][3], base;
  auto set = [](double* v, double p, double q, double r) { v[0] = p; v[1] = q; v[2] = r; };
  auto setm = [](double m[3][3], double a0, double a1, double a2, double b0, double b1, double b2,
                 double c0, double c1, double c2) {
    m[0][0] = a0; m[0][1] = a1; m[0][2] = a2; m[1][0] = b0; m[1][1] = b1; m[1][2] = b2;
    m[2][0] = c0; m[2][1] = c1; m[2][2] = c2;
  };
  if (i == 0) {
    if (j == 0) { set(a, x.tb, x.bs, x.bq); set(b, x.tb, x.bs, x.bq);
      setm(m, x.t2, x.ts, x.tq, x.ts, x.s2, x.sq, x.tq, x.sq, x.q2); base = x.b2; }
    else if (j == 1) { set(a, x.ts, x.s2, x.sq); set(b, x.tb, x.b2, x.bq);
      setm(m, x.t2, x.ts, x.tq, x.tb, x.bs, x.bq, x.tq, x.sq, x.q2); base = x.bs; }
    else { set(a, x.tq, x.sq, x.q2); set(b, x.tb, x.b2, x.bs);
      setm(m, x.t2, x.ts, x.tq, x.tb, x.bs, x.bq, x.ts, x.s2, x.sq); base = x.bq; }
  } else if (i == 1) {
    if (j == 0) { set(a, x.tb, x.b2, x.bq); set(b, x.ts, x.s2, x.sq);
      setm(m, x.t2, x.tb, x.tq, x.ts, x.bs, x.sq, x.tq, x.bq, x.q2); base = x.bs; }
    else if (j == 1) { set(a, x.ts, x.bs, x.sq); set(b, x.ts, x.bs, x.sq);
      setm(m, x.t2, x.tb, x.tq, x.tb, x.b2, x.bq, x.tq, x.bq, x.q2); base = x.s2; }
    else { set(a, x.tq, x.bq, x.q2); set(b, x.ts, x.bs, x.s2);
      setm(m, x.t2, x.tb, x.tq, x.tb, x.b2, x.bq, x.ts, x.bs, x.sq); base = x.sq; }
  } else {
    if (j == 0) { set(a, x.tb, x.b2, x.bs); set(b, x.tq, x.sq, x.q2);
      setm(m, x.t2, x.tb, x.ts, x.ts, x.bs, x.s2, x.tq, x.bq, x.sq); base = x.bq; }
    else if (j == 1) { set(a, x.ts, x.bs, x.s2); set(b, x.tq, x.bq, x.q2);
      setm(m, x.t2, x.tb, x.ts, x.tb, x.b2, x.bs, x.tq, x.bq, x.sq); base = x.sq; }
    else { set(a, x.tq, x.bq, x.sq); set(b, x.tq, x.bq, x.sq);
      setm(m, x.t2, x.tb, x.ts, x.tb, x.b2, x.bs, x.ts, x.bs, x.s2); base = x.q2; }
  }
  return base - aTmb(a, m, b);
}
// G = H^-1 of the (T, muB, muS, muQ) Hessian of p over the directions that
// are not decoupled-and-frozen (an all-zero row), Gauss-Jordan with partial
// pivoting; the conformal-diagonal model's cross terms are its exact zeros.
void exact_hessian_inverse(const Chi& X, bool diag, double G[4][4]) {
  double H[4][4] = {{X.t2, X.tb, X.ts, X.tq}, {X.tb, X.b2, X.bs, X.bq},
                    {X.ts, X.bs, X.s2, X.sq}, {X.tq, X.bq, X.sq, X.q2}};
  if (diag)
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) if (i != j) H[i][j] = 0.0;
  int keep[4], m = 0;
  for (int i = 0; i < 4; i++) {
    bool zero = true;
    for (int j = 0; j < 4; j++) zero = zero && (H[i][j] == 0.0);
    if (!zero) keep[m++] = i;
  }
  double A[4][8] = {{0}};
  for (int i = 0; i < m; i++) {
    for (int j = 0; j < m; j++) A[i][j] = H[keep[i]][keep[j]];
    A[i][m + i] = 1.0;
  }
  for (int col = 0; col < m; col++) {
    int p = col;
    for (int r = col + 1; r < m; r++) if (std::fabs(A[r][col]) > std::fabs(A[p][col])) p = r;
    if (p != col) for (int j = 0; j < 2 * m; j++) std::swap(A[col][j], A[p][j]);
    const double piv = A[col][col];
    for (int j = 0; j < 2 * m; j++) A[col][j] /= piv;
    for (int r = 0; r < m; r++) {
      if (r == col || A[r][col] == 0.0) continue;
      const double f = A[r][col];
      for (int j = 0; j < 2 * m; j++) A[r][j] -= f * A[col][j];
    }
  }
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) G[i][j] = 0.0;
  for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) G[keep[i]][keep[j]] = A[i][m + j];
}
}  // namespace

// include/eos.h:121-175 (set_thermo) restricted to the fields the hot path
// reads, with dw/ds, dw/drho_X from src/eos.cpp:276-344.
void eos_set_thermo(const Config& c, const Table* tab, int k, const double x[4], double th[16]) {
  double o[17];
  model_thermo(c, tab, chain_model(c, k), x, o);
  const int rm = frozen_mode(tab, chain_model(c, k));
  const double T = x[0], mB = x[1], mQ = x[2], mS = x[3];
  const double p = o[0], s = o[1], B = o[2], S = o[3], Q = o[4], e = o[5];
  Chi X{o[16], o[13], o[14], o[15], o[7], o[8], o[9], o[10], o[11], o[12]};
  th[kT] = T; th[kMuB] = mB; th[kMuS] = mS; th[kMuQ] = mQ;
  th[kP] = p; th[kS] = s; th[kRhoB] = B; th[kRhoS] = S; th[kRhoQ] = Q; th[kE] = e;
  th[kW] = e + p; th[kCs2] = o[6];
  const bool hB = std::fabs(B) > kTiny, hS = std::fabs(S) > kTiny, hQ = std::fabs(Q) > kTiny;
  if (c.thermo_mode == 1) {
    // Exact form: G = H^-1 over the (T, muB, muS, muQ) directions that are not
    // decoupled-and-frozen (an all-zero Hessian row), with the cross terms of
    // the conformal-diagonal model taken as the exact zeros its p(T, mu) has.
    // dw/ds|rho = T + s G_TT + sum_a rho_a G_aT, dw/drho_a = mu_a + s G_Ta +
    // sum_b rho_b G_ba, charge terms gated by |rho| > TINY as in the reference.
    double G[4][4];
    exact_hessian_inverse(X, chain_model(c, k) == mConfDiag, G);
    const double rho[4] = {0.0, B, S, Q};
    const bool act[4] = {true, hB, hS, hQ};
    const double mu[4] = {T, mB, mS, mQ};
    double dw[4];
    for (int a = 0; a < 4; a++) {
      if (a > 0 && !act[a]) { dw[a] = mu[a]; continue; }
      double acc = mu[a] + s * G[0][a];
      for (int b = 1; b < 4; b++) if (act[b]) acc += rho[b] * G[b][a];
      dw[a] = acc;
    }
    th[kDwds] = dw[0]; th[kDwdB] = dw[1]; th[kDwdS] = dw[2]; th[kDwdQ] = dw[3];
    return;
  }
  double ct = 0.0;
  if (hB) ct += B / term2(X, 0, rm);
  if (hQ) ct += Q / term2(X, 2, rm);
  if (hS) ct += S / term2(X, 1, rm);
  th[kDwds] = T + s / term1(X, rm) + ct;
  ct = 0.0;
  if (hB) {
    ct += s / term3(X, 0, rm) + B / term4(X, 0, 0, rm);
    if (hQ) ct += Q / term4(X, 0, 2, rm);
    if (hS) ct += S / term4(X, 0, 1, rm);
  }
  th[kDwdB] = mB + ct;
  ct = 0.0;
  if (hS) {
    ct += s / term3(X, 1, rm) + S / term4(X, 1, 1, rm);
    if (hB) ct += B / term4(X, 1, 0, rm);
    if (hQ) ct += Q / term4(X, 1, 2, rm);
  }
  th[kDwdS] = mS + ct;
  ct = 0.0;
  if (hQ) {
    ct += s / term3(X, 2, rm) + Q / term4(X, 2, 2, rm);
    if (hB) ct += B / term4(X, 2, 0, rm);
    if (hS) ct += S / term4(X, 2, 1, rm);
  }
  th[kDwdQ] = mQ + ct;
}

// The twelve derivatives of alpha_a = mu_a / T at fixed (s, rho) that the
// diffusion sector reads (src/eos.cpp:337-493, dalpha_Bds .. dalpha_QdQ).
// out[a] = dalpha_a/ds, out[3 + 3a + b] = dalpha_a/drho_b, charges a, b in
// the order B, S, Q. The reference chain (thermo_mode 0) uses
// dalpha_a/ds = -mu_a/T^2 / (ds/dT) + [rho_a] 1/T / (ds/dmu_a) and
// dalpha_a/drho_b = [rho_b] (-mu_a/T^2 / (drho_b/dT) + [rho_a] 1/T / (drho_b/dmu_a)),
// [rho] meaning |rho| > TINY, with its operation order (dalpha_BdB adds the
// 1/T term first). The exact form (thermo_mode 1) replaces 1/(dx/dy) by the
// entries of H^-1 under the same gates.
void eos_alpha_derivs(const Config& c, const Table* tab, int k, const double x[4], double out[12]) {
  double o[17];
  model_thermo(c, tab, chain_model(c, k), x, o);
  const int rm = frozen_mode(tab, chain_model(c, k));
  const double T = x[0];
  const double mu[3] = {x[1], x[3], x[2]};            // muB, muS, muQ
  const double rho[3] = {o[2], o[3], o[4]};           // B, S, Q
  const Chi X{o[16], o[13], o[14], o[15], o[7], o[8], o[9], o[10], o[11], o[12]};
  bool h[3];
  for (int a = 0; a < 3; a++) h[a] = std::fabs(rho[a]) > kTiny;
  if (c.thermo_mode == 1) {
    double G[4][4];
    exact_hessian_inverse(X, chain_model(c, k) == mConfDiag, G);
    // H index: 0 T, 1 B, 2 S, 3 Q
    for (int a = 0; a < 3; a++) {
      double ct = 0.0;
      if (h[a]) ct += 1 / T * G[a + 1][0];
      out[a] = -mu[a] / T / T * G[0][0] + ct;
      for (int b = 0; b < 3; b++) {
        double v = 0.0;
        if (h[b]) {
          v += -mu[a] / T / T * G[0][b + 1];
          if (h[a]) v += 1 / T * G[a + 1][b + 1];
        }
        out[3 + 3 * a + b] = v;
      }
    }
    return;
  }
  for (int a = 0; a < 3; a++) {
    double ct = 0.0;
    if (h[a]) ct += 1 / T / term2(X, a, rm);
    out[a] = -mu[a] / T / T / term1(X, rm) + ct;
    for (int b = 0; b < 3; b++) {
      double v = 0.0;
      if (h[b]) {
        if (a == b && a == 0) {
          v += 1 / T / term4(X, b, a, rm) - mu[a] / T / T / term3(X, b, rm);
        } else {
          v += -mu[a] / T / T / term3(X, b, rm);
          if (h[a]) v += 1 / T / term4(X, b, a, rm);
        }
      }
      out[3 + 3 * a + b] = v;
    }
  }
}

}  // namespace orc
