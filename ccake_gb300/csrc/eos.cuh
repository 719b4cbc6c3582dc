// Device equation of state: analytic conformal / conformal-diagonal models,
// the tabulated 4-D EoS with multilinear lookup, the (e|s, B, S, Q) ->
// (T, muB, muQ, muS) Newton root finder with the reference's seed chain, and
// the enthalpy derivatives dw/ds, dw/drho. Everything is FP64.
#pragma once
#include "common.cuh"

namespace ccake {

// Model scales with their reciprocals (the FP64 pipe is the bottleneck, so
// the models multiply by 1/T0 instead of dividing by T0).
struct Scales {
  double c, T0, muB0, muQ0, muS0;
  double iT0, iB0, iQ0, iS0;
  double ic4;   // 1 / (4 c T0^4), of the analytic inverses
};
__host__ __device__ inline Scales make_scales(double c, double T0, double muB0, double muQ0, double muS0) {
  return Scales{c, T0, muB0, muQ0, muS0, 1.0 / T0, 1.0 / muB0, 1.0 / muQ0, 1.0 / muS0,
                1.0 / (4.0 * c * T0 * T0 * T0 * T0)};
}

// Tabulated EoS in device memory: uniform (T, muB, muQ, muS) grid, muS
// fastest, 17 fields per node (p s B S Q e cs2 chiBB chiQQ chiSS chiBQ chiBS
// chiQS chiTB chiTQ chiTS chiTT), layout of reference src/eos_table.cpp:31-35.
struct TableView {
  const double* f = nullptr;
  // FP32 copy of the densities s, rhoB, rhoS, rhoQ, e of every node (8 floats
  // a node, the last 3 zero), for the FP32 Newton Jacobian of the mixed form
  const float* fd = nullptr;
  int n[4] = {1, 1, 1, 1};
  double lo[4] = {0, 0, 0, 0};
  double d[4] = {0, 0, 0, 0};
  double id[4] = {0, 0, 0, 0};   // 1 / d, rounded on the host (mixed-form lookup)
};

// Pre-inverted (s, rhoB, rhoS, rhoQ) -> thermodynamics tables, the
// reference's EoS_Interpolator (include/eos_interpolator.h:33-165,
// src/eos_interpolator.cpp:531-739): one tile a decade of each density,
// tiles of N^4 nodes at x = min + i * step (min = 10^e, step = 10^(e+1) / N,
// utilities/generate_eos_table.cpp:196-203), 11 values a node in the order of
// kPreVars, nodes row-major with rhoQ fastest.
constexpr int kPreMaxTiles = 8;
enum PreVar : int { PV_T = 0, PV_MUB, PV_MUQ, PV_MUS, PV_E, PV_P, PV_CS2, PV_DWDS, PV_DWDB, PV_DWDQ, PV_DWDS_S, kPreVars };
struct PreinvView {
  const double* v = nullptr;             // [tile][node][kPreVars]
  int nt[4] = {0, 0, 0, 0};              // tiles on each axis (s, rhoB, rhoS, rhoQ)
  int N = 0;                             // nodes on each axis of a tile
  int e_lo[4] = {0, 0, 0, 0};            // decade exponent of tile 0
  double mn[4][kPreMaxTiles];            // tile minimum, 10^e (host pow)
  double st[4][kPreMaxTiles];            // tile step, 10^(e+1) / N
};

struct EosDev {
  int kind;                 // ccake_config::eos_kind
  int thermo_mode;          // 0 reference chain, 1 exact Hessian inverse
  Scales own;               // scales of the analytic default model
  Scales conf, cdiag;       // fallback scales behind a table
  TableView tab;
  // 1: Newton Jacobians of the table in FP32 (residuals stay FP64)
  int jac32 = 0;
  // restrict_mu_T_ratios: table solutions with a chemical potential above
  // 3.5 T are refused (src/eos.cpp:781-786)
  int restrict_mu_T = 0;
  // device copy of the pre-inverted tables' description; non-null: the step's
  // thermodynamics come from the tables instead of the inversion
  const PreinvView* pre = nullptr;
};

enum Model : int { M_CONF = 0, M_CDIAG = 1, M_TABLE = 2, M_TANH = 3 };

// Chains of the reference (src/eos_initialization.cpp:216-501):
// conformal -> [conformal, conformal_diagonal]; conformal_diagonal -> [itself];
// table -> [table, tanh_conformal, conformal, conformal_diagonal] (the tanh
// stage with use_tanh_conformal = true, include/eos_header.h:7).
__host__ __device__ inline int chain_len(int kind) { return kind == 0 ? 2 : (kind == 1 ? 1 : 4); }
__host__ __device__ inline int chain_model(int kind, int k) {
  if (kind == 0) return k == 0 ? M_CONF : M_CDIAG;
  if (kind == 1) return M_CDIAG;
  return k == 0 ? M_TABLE : (k == 1 ? M_TANH : (k == 2 ? M_CONF : M_CDIAG));
}
// The tanh-conformal fallback shares the conformal fallback's scales: the
// reference derives both from the table by the same rule
// (src/eos_initialization.cpp:276-341 and :343-403).
__host__ __device__ inline Scales model_scales(const EosDev& e, int model) {
  if (e.kind == 2 && model != M_TABLE) return model == M_CDIAG ? e.cdiag : e.conf;
  return e.own;
}

// p = c T0^4 x^2, x = (T/T0)^2 + sum (mu/mu0)^2 (reference include/eos_conformal.h:33-194).
__host__ __device__ inline void conformal_thermo(const Scales& k, const double* x4, double* o) {
  const double T = x4[0], mB = x4[1], mQ = x4[2], mS = x4[3];
  const double iT = k.iT0, iB = k.iB0, iQ = k.iQ0, iS = k.iS0;
  const double iT2 = iT * iT, iB2 = iB * iB, iQ2 = iQ * iQ, iS2 = iS * iS;
  const double x = T * T * iT2 + mB * mB * iB2 + mS * mS * iS2 + mQ * mQ * iQ2;
  const double cp = k.c * k.T0 * k.T0 * k.T0 * k.T0;
  const double p = cp * x * x;
  const double s = 4.0 * cp * T * x * iT2;
  const double B = 4.0 * cp * mB * x * iB2;
  const double S = 4.0 * cp * mS * x * iS2;
  const double Q = 4.0 * cp * mQ * x * iQ2;
  o[0] = p; o[1] = s; o[2] = B; o[3] = S; o[4] = Q;
  o[5] = (s * T + mB * B + mQ * Q + mS * S) - p;
  o[6] = 1.0 / 3.0;
  o[7] = cp * (8.0 * mB * mB * iB2 * iB2 + 4.0 * x * iB2);
  o[8] = cp * (8.0 * mQ * mQ * iQ2 * iQ2 + 4.0 * x * iQ2);
  o[9] = cp * (8.0 * mS * mS * iS2 * iS2 + 4.0 * x * iS2);
  o[10] = 8.0 * cp * mB * mQ * iB2 * iQ2;
  o[11] = 8.0 * cp * mB * mS * iB2 * iS2;
  o[12] = 8.0 * cp * mS * mQ * iS2 * iQ2;
  o[13] = 8.0 * cp * T * mB * iT2 * iB2;
  o[14] = 8.0 * cp * T * mQ * iT2 * iQ2;
  o[15] = 8.0 * cp * T * mS * iT2 * iS2;
  o[16] = cp * (8.0 * T * T * iT2 * iT2 + 4.0 * x * iT2);
}

// p = c T0^4 [(T/T0)^4 + sum (mu/mu0)^4]; cross susceptibilities are the
// TINY placeholders of the reference (include/eos_conformal_diagonal.h:78-205).
__host__ __device__ inline void confdiag_thermo(const Scales& k, const double* x4, double* o) {
  const double T = x4[0], mB = x4[1], mQ = x4[2], mS = x4[3];
  const double cp = k.c * k.T0 * k.T0 * k.T0 * k.T0;
  const double rT = T * k.iT0, rB = mB * k.iB0, rQ = mQ * k.iQ0, rS = mS * k.iS0;
  const double p = cp * (rT * rT * rT * rT + rB * rB * rB * rB + rS * rS * rS * rS + rQ * rQ * rQ * rQ);
  const double s = 4.0 * cp * rT * rT * rT * k.iT0;
  const double B = 4.0 * cp * rB * rB * rB * k.iB0;
  const double S = 4.0 * cp * rS * rS * rS * k.iS0;
  const double Q = 4.0 * cp * rQ * rQ * rQ * k.iQ0;
  o[0] = p; o[1] = s; o[2] = B; o[3] = S; o[4] = Q;
  o[5] = (s * T + mB * B + mQ * Q + mS * S) - p;
  o[6] = 1.0 / 3.0;
  o[7] = 12.0 * cp * rB * rB * (k.iB0 * k.iB0);
  o[8] = 12.0 * cp * rQ * rQ * (k.iQ0 * k.iQ0);
  o[9] = 12.0 * cp * rS * rS * (k.iS0 * k.iS0);
  for (int i = 10; i < 16; i++) o[i] = kTiny;
  o[16] = 12.0 * cp * rT * rT * (k.iT0 * k.iT0);
}

// The tanh-modulated conformal model (include/eos_tanh_conformal.h): the
// conformal pressure p_c of the given scales times
// t(T) = (1 + tanh((T - Tc)/Ts)) / 2 with Tc = 220 MeV and Ts = 120 MeV
// (src/eos_initialization.cpp:334-335). Densities and susceptibilities follow
// from p = t p_c by the product rule (t' = sech^2((T - Tc)/Ts) / (2 Ts),
// t'' = -2 tanh((T - Tc)/Ts) t' / Ts). Its c_s^2 is the adiabatic speed of
// sound, dp/de at fixed ratios s : rhoB : rhoS : rhoQ. Along dn = n dlambda
// (n = (s, rho) = grad p, chi = the Hessian of p in (T, mu)) one has
// dp = n . chi^-1 n dlambda and de = T ds + mu . drho = w dlambda, so
// c_s^2 = n . chi^-1 n / w with w = T s + mu . rho.
constexpr double kTanhTc = 220.0 / kHbarcMeVfm, kTanhTs = 120.0 / kHbarcMeVfm;

template <class R>
__host__ __device__ inline void solve4(R A[4][4], R* b, R* x);

// cs2 = false leaves o[6] unset (the Newton iterations read the densities
// and the susceptibilities only; the 4x4 solve is for c_s^2).
__host__ __device__ inline void tanh_conformal_thermo(const Scales& k, const double* x4, double* o, bool cs2 = true) {
  double c[17];
  conformal_thermo(k, x4, c);
  const double T = x4[0], mB = x4[1], mQ = x4[2], mS = x4[3];
  const double y = (T - kTanhTc) / kTanhTs;
  const double th = tanh(y), sc = 1.0 / cosh(y);
  const double t = 0.5 * (1.0 + th);
  const double tp = 0.5 * sc * sc / kTanhTs;
  const double tpp = -2.0 * th * tp / kTanhTs;
  const double p = t * c[0], s = t * c[1] + tp * c[0];
  const double B = t * c[2], S = t * c[3], Q = t * c[4];
  o[0] = p; o[1] = s; o[2] = B; o[3] = S; o[4] = Q;
  o[5] = (s * T + mB * B + mQ * Q + mS * S) - p;
  for (int i = 7; i <= 12; i++) o[i] = t * c[i];
  o[13] = t * c[13] + tp * c[2];
  o[14] = t * c[14] + tp * c[4];
  o[15] = t * c[15] + tp * c[3];
  o[16] = t * c[16] + 2.0 * tp * c[1] + tpp * c[0];
  if (!cs2) return;
  // c_s^2 = n . chi^-1 n / w, n and chi in (T, muB, muQ, muS) order
  double H[4][4] = {{o[16], o[13], o[14], o[15]},
                    {o[13], o[7], o[10], o[11]},
                    {o[14], o[10], o[8], o[12]},
                    {o[15], o[11], o[12], o[9]}};
  double n[4] = {s, B, Q, S}, r[4] = {s, B, Q, S}, z[4];
  solve4<double>(H, r, z);
  const double w = s * T + mB * B + mQ * Q + mS * S;
  o[6] = (n[0] * z[0] + n[1] * z[1] + n[2] * z[2] + n[3] * z[3]) / w;
}

// Multilinear lookup with the reference's index rule (src/interpolatorND.cpp:250-317):
// integer part by truncation toward zero, last cell reused at the upper edge,
// NaN outside.
// jac (optional): derivatives of the interpolated s, rhoB, rhoS, rhoQ, e
// (fields 1..5) with respect to (T, muB, muQ, muS), the exact Jacobian of the
// multilinear interpolant inside the cell.
__host__ __device__ inline void table_thermo(const TableView& t, const double* x, double* o,
                                             double (*jac)[4] = nullptr) {
  int ind[4];
  double fr[4], dfr[4];
  for (int k = 0; k < 4; k++) {
    if (isnan(x[k])) { for (int i = 0; i < 17; i++) o[i] = NAN; return; }
    if (t.n[k] <= 1 || fabs(t.d[k]) < 1e-30) { ind[k] = 0; fr[k] = 1.0; dfr[k] = 0.0; continue; }
    const double q = (x[k] - t.lo[k]) / t.d[k];
    const double ip = trunc(q);
    fr[k] = 1.0 - (q - ip);
    dfr[k] = -1.0 / t.d[k];
    ind[k] = (int)ip;
    if (ind[k] + 1 == t.n[k]) { fr[k] = 1.0 - fr[k]; dfr[k] = -dfr[k]; ind[k]--; }
    if (ind[k] < 0 || ind[k] >= t.n[k] || !(fabs(q) < 2e9)) { for (int i = 0; i < 17; i++) o[i] = NAN; return; }
  }
  // with a Jacobian (the Newton iterations) only the densities o[1..5] are
  // formed: the other fields are not read there
  if (jac) for (int i = 1; i < 6; i++) o[i] = 0.0;
  else for (int i = 0; i < 17; i++) o[i] = 0.0;
  if (jac)
    for (int f = 0; f < 5; f++) for (int j = 0; j < 4; j++) jac[f][j] = 0.0;
  for (int h = 0; h < 16; h++) {
    const int b[4] = {(h >> 3) & 1, (h >> 2) & 1, (h >> 1) & 1, h & 1};
    double wk[4], w = 1.0;
    long idx = 0;
    for (int k = 0; k < 4; k++) {
      wk[k] = fr[k] + b[k] - 2.0 * b[k] * fr[k];
      w *= wk[k];
      const int c = (t.n[k] <= 1) ? 0 : ind[k] + b[k];
      idx = idx * t.n[k] + c;
    }
    const double* node = t.f + (size_t)idx * 17;
    if (jac) {
      for (int j = 0; j < 4; j++) {
        double dw = (1.0 - 2.0 * b[j]) * dfr[j];
        for (int k = 0; k < 4; k++)
          if (k != j) dw *= wk[k];
        for (int f = 0; f < 5; f++) jac[f][j] += dw * node[1 + f];
      }
      for (int i = 1; i < 6; i++) o[i] += w * node[i];
    } else {
      for (int i = 0; i < 17; i++) o[i] += w * node[i];
    }
  }
}

// The same multilinear lookup for the mixed form (EosDev::jac32): cell
// fractions from the host-rounded inverse spacings (a multiplication instead
// of a division), the 16 corner weights as products of two pair products,
// and, with jac, the Jacobian of the densities in FP32 from the FP32 node
// copy; the interpolated values stay FP64. It differs from table_thermo by
// roundings of the weights only (relative 1e-16).
__host__ __device__ inline void table_thermo_fast(const TableView& t, const double* x, double* o,
                                                  float (*jac)[4] = nullptr) {
  int ind[4];
  double fr[4];
  float dfrf[4];
  for (int k = 0; k < 4; k++) {
    if (isnan(x[k])) { for (int i = 0; i < 17; i++) o[i] = NAN; return; }
    if (t.n[k] <= 1 || fabs(t.d[k]) < 1e-30) { ind[k] = 0; fr[k] = 1.0; dfrf[k] = 0.0f; continue; }
    const double q = (x[k] - t.lo[k]) * t.id[k];
    const double ip = trunc(q);
    fr[k] = 1.0 - (q - ip);
    dfrf[k] = -(float)t.id[k];
    ind[k] = (int)ip;
    if (ind[k] + 1 == t.n[k]) { fr[k] = 1.0 - fr[k]; dfrf[k] = -dfrf[k]; ind[k]--; }
    if (ind[k] < 0 || ind[k] >= t.n[k] || !(fabs(q) < 2e9)) { for (int i = 0; i < 17; i++) o[i] = NAN; return; }
  }
  // corner h = (b0 b1 b2 b3): weight p01[b0 b1] * p23[b2 b3]; node offset
  // from the lower corner by the row-major strides (0 on a single-node axis)
  double w1[4];
  for (int k = 0; k < 4; k++) w1[k] = 1.0 - fr[k];
  const double p01[4] = {fr[0] * fr[1], fr[0] * w1[1], w1[0] * fr[1], w1[0] * w1[1]};
  const double p23[4] = {fr[2] * fr[3], fr[2] * w1[3], w1[2] * fr[3], w1[2] * w1[3]};
  long st[4], base = 0;
  {
    long s = 1;
    for (int k = 3; k >= 0; k--) {
      st[k] = (t.n[k] <= 1) ? 0 : s;
      base += (long)ind[k] * s;
      s *= t.n[k];
    }
  }
  const int i0 = jac ? 1 : 0, i1 = jac ? 6 : 17;
  for (int i = i0; i < i1; i++) o[i] = 0.0;
  float frf[4], w1f[4];
  if (jac) {
    for (int k = 0; k < 4; k++) { frf[k] = (float)fr[k]; w1f[k] = 1.0f - frf[k]; }
    for (int f = 0; f < 5; f++) for (int j = 0; j < 4; j++) jac[f][j] = 0.0f;
  }
  for (int h = 0; h < 16; h++) {
    const int b[4] = {(h >> 3) & 1, (h >> 2) & 1, (h >> 1) & 1, h & 1};
    const double w = p01[h >> 2] * p23[h & 3];
    const long idx = base + b[0] * st[0] + b[1] * st[1] + b[2] * st[2] + b[3] * st[3];
    const double* node = t.f + (size_t)idx * 17;
    if (jac) {
      for (int i = 1; i < 6; i++) o[i] += w * node[i];
      const float* nd = t.fd + (size_t)idx * 8;
      float wk[4];
      for (int k = 0; k < 4; k++) wk[k] = b[k] ? w1f[k] : frf[k];
      for (int j = 0; j < 4; j++) {
        float dw = b[j] ? -dfrf[j] : dfrf[j];
        for (int k = 0; k < 4; k++)
          if (k != j) dw *= wk[k];
        for (int f = 0; f < 5; f++) jac[f][j] += dw * nd[f];
      }
    } else {
      for (int i = 0; i < 17; i++) o[i] += w * node[i];
    }
  }
}

__host__ __device__ inline void model_thermo(const EosDev& e, int model, const double* x4, double* o) {
  if (model == M_TABLE) {
    if (e.jac32 && e.tab.fd) table_thermo_fast(e.tab, x4, o);
    else table_thermo(e.tab, x4, o);
    return;
  }
  const Scales k = model_scales(e, model);
  if (model == M_CONF) conformal_thermo(k, x4, o);
  else if (model == M_TANH) tanh_conformal_thermo(k, x4, o);
  else confdiag_thermo(k, x4, o);
}

__host__ __device__ inline void model_box(const EosDev& e, int model, double* lo, double* hi) {
  if (model == M_TABLE) {
    for (int k = 0; k < 4; k++) { lo[k] = e.tab.lo[k]; hi[k] = e.tab.lo[k] + e.tab.d[k] * (e.tab.n[k] - 1); }
    return;
  }
  lo[0] = 0.0; hi[0] = kTbqsInf;
  for (int i = 1; i < 4; i++) { lo[i] = -kTbqsInf; hi[i] = kTbqsInf; }
}

// Densities (e|s, B, Q, S) at x = (T, muB, muQ, muS) and their Jacobian: the
// Hessian of p (exactly diagonal for the conformal-diagonal model).
// For the table the Jacobian is that of the interpolated densities (the
// function the solver zeroes; the reference's GSL hybrids solver
// differentiates it by finite differences), not the interpolated
// susceptibilities.
// Jf (mixed form, table model): the Jacobian in FP32 instead of J.
// Reduced modes of the reference for a model whose chemical-potential axes
// are frozen (a table with one node along them). Derivatives
// (src/eos.cpp:129-141): 2 every mu frozen (T-only), 1 muQ and muS frozen
// (baryon-only), else 0. Root finder (src/rootfinder.cpp:447-491): the same,
// and only with zero target charges (T-only: B, Q, S; baryon-only: Q, S).
__host__ __device__ inline int frozen_mode(const EosDev& e, int model) {
  if (model != M_TABLE) return 0;
  const bool fb = e.tab.n[1] <= 1, fq = e.tab.n[2] <= 1, fs = e.tab.n[3] <= 1;
  if (fb && fq && fs) return 2;
  return (fq && fs) ? 1 : 0;
}
__host__ __device__ inline int root_mode(const EosDev& e, int model, const double* tgt) {   // (e|s, B, Q, S)
  if (model != M_TABLE) return 0;
  const bool fb = e.tab.n[1] <= 1, fq = e.tab.n[2] <= 1, fs = e.tab.n[3] <= 1;
  const bool zb = fabs(tgt[1]) < 1e-30, zq = fabs(tgt[2]) < 1e-30, zs = fabs(tgt[3]) < 1e-30;
  if (fb && fq && fs && zb && zq && zs) return 2;
  return (fq && fs && zq && zs) ? 1 : 0;
}

// rmode: in a reduced mode the equations of the frozen chemical potentials
// are mu = 0 (src/rootfinder.cpp:119-140; their targets are 0).
__host__ __device__ inline void dens_jac(const EosDev& e, int model, int entropy, const double* x, double* f,
                                         double J[4][4], float (*Jf)[4] = nullptr, int rmode = 0) {
  double o[17];
  if (model == M_TABLE && Jf) {
    float jac[5][4];
    table_thermo_fast(e.tab, x, o, jac);
    f[0] = entropy ? o[1] : o[5];
    f[1] = o[2];
    f[2] = o[4];
    f[3] = o[3];
    for (int j = 0; j < 4; j++) {
      Jf[0][j] = entropy ? jac[0][j] : jac[4][j];
      Jf[1][j] = jac[1][j];
      Jf[2][j] = jac[3][j];
      Jf[3][j] = jac[2][j];
    }
    for (int i = (rmode == 2 ? 1 : 2); rmode && i < 4; i++) {
      f[i] = x[i];
      for (int j = 0; j < 4; j++) Jf[i][j] = (i == j) ? 1.0f : 0.0f;
    }
    return;
  }
  if (model == M_TABLE) {
    double jac[5][4];
    table_thermo(e.tab, x, o, jac);
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
    for (int i = (rmode == 2 ? 1 : 2); rmode && i < 4; i++) {
      f[i] = x[i];
      for (int j = 0; j < 4; j++) J[i][j] = (i == j) ? 1.0 : 0.0;
    }
    return;
  }
  if (model == M_TANH) tanh_conformal_thermo(model_scales(e, model), x, o, false);
  else model_thermo(e, model, x, o);
  double H[4][4];
  if (model == M_CDIAG) {
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
#pragma unroll
  for (int j = 0; j < 4; j++) {
    J[1][j] = H[1][j];
    J[2][j] = H[2][j];
    J[3][j] = H[3][j];
    J[0][j] = entropy ? H[0][j] : x[0] * H[0][j] + x[1] * H[1][j] + x[2] * H[2][j] + x[3] * H[3][j];
  }
}

// 4x4 solve, partial pivoting; a zero pivot leaves its unknown unchanged.
template <class R>
__host__ __device__ inline void solve4(R A[4][4], R* b, R* x) {
  bool dead[4] = {false, false, false, false};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    int p = k;
    R best = fabs(A[k][k]);
    for (int i = k + 1; i < 4; i++)
      if (fabs(A[i][k]) > best) { best = fabs(A[i][k]); p = i; }
    if (p != k) {
      for (int j = 0; j < 4; j++) { R tmp = A[k][j]; A[k][j] = A[p][j]; A[p][j] = tmp; }
      R tb = b[k]; b[k] = b[p]; b[p] = tb;
    }
    if (A[k][k] == R(0)) { dead[k] = true; continue; }
    for (int i = k + 1; i < 4; i++) {
      if (A[i][k] == R(0)) continue;
      const R m = A[i][k] / A[k][k];
      for (int j = k; j < 4; j++) A[i][j] -= m * A[k][j];
      b[i] -= m * b[k];
    }
  }
#pragma unroll
  for (int k = 3; k >= 0; k--) {
    if (dead[k]) { x[k] = R(0); continue; }
    R acc = b[k];
    for (int j = k + 1; j < 4; j++) acc -= A[k][j] * x[j];
    x[k] = acc / A[k][k];
  }
}

// One Newton attempt from a seed. Stopping rule: the reference's max|F| < 1e-10
// (include/rootfinder.h:36-37); then full steps (at most 8) until the largest
// relative step is below 1e-12. 100 iterations at most; damped by residual
// halving; leaving the model box fails.
__host__ __device__ inline bool newton_attempt(const EosDev& e, int model, int entropy, const double* tgt,
                                               const double* lo, const double* hi, double* x, int* iters,
                                               int max_it = 100, int rmode = 0) {
  // f, J at the current x are carried over from the accepted trial point of
  // the previous iteration (the same values a fresh evaluation would give),
  // so an undamped iteration costs one density/Jacobian evaluation.
  int extra = -1, nslow1 = 0, nslow2 = 0;
  double f[4], J[4][4], xgood[4] = {0.0, 0.0, 0.0, 0.0};
  // mixed form, table model: FP32 Jacobian and Newton step (the residual,
  // its tests and the iterate stay FP64)
  const bool f32 = e.jac32 && model == M_TABLE && e.tab.fd;
  float Jf[4][4];
  bool have = false;
  const bool diag = (model == M_CDIAG);
  for (int it = 0; it < max_it; it++) {
    if (!have) dens_jac(e, model, entropy, x, f, J, f32 ? Jf : nullptr, rmode);
    have = false;
    // the largest |F_i|, NaN if any is NaN: a non-finite residual fails the
    // attempt, as GSL_EBADFUNC fails the reference's solver
    double F[4], fres = 0.0;
    for (int i = 0; i < 4; i++) {
      F[i] = f[i] - tgt[i];
      const double a = fabs(F[i]);
      fres = (a > fres || a != a) ? a : fres;
    }
    if (!(fres <= 1e300)) { *iters += it + 1; return false; }
    if (extra < 0 && fres < 1e-10) extra = 0;
    double dx[4];
    if (diag) {
      // the conformal-diagonal Jacobian is diagonal: the 4x4 elimination
      // reduces to these divisions (a zero pivot leaves its unknown unchanged)
      for (int i = 0; i < 4; i++) dx[i] = (J[i][i] == 0.0) ? 0.0 : (-F[i]) / J[i][i];
    } else if (f32) {
      float rhs[4] = {(float)-F[0], (float)-F[1], (float)-F[2], (float)-F[3]}, dxf[4];
      solve4(Jf, rhs, dxf);
      for (int i = 0; i < 4; i++) dx[i] = dxf[i];
    } else {
      double rhs[4] = {-F[0], -F[1], -F[2], -F[3]};
      solve4(J, rhs, dx);
    }
    if (extra >= 0) {
      // x met the residual test. Full steps continue (at most 8) until the
      // relative step is below 1e-12; each is verified at the next iteration
      // and, if its residual left the tolerance, the last verified point is
      // returned (the point the reference's solver stops at).
      if (extra > 0 && !(fres < 1e-10)) {
        for (int i = 0; i < 4; i++) x[i] = xgood[i];
        *iters += it;
        return true;
      }
      double y[4], rel = 0.0;
      bool inbox = true;
      for (int i = 0; i < 4; i++) {
        xgood[i] = x[i];
        y[i] = x[i] + dx[i];
        const double r = fabs(dx[i]) / fmax(fabs(x[i]), 1e-300);
        rel = rel > r ? rel : r;
        // every iterate stays in the model's box (src/rootfinder.cpp:277-330)
        inbox = inbox && (y[i] >= lo[i] && y[i] <= hi[i]);
      }
      const bool usable = y[0] > 0 && isfinite(y[0]) && inbox;
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
    double lam = 1.0, y[4];
    for (int h = 0; h < 7; h++) {
      for (int i = 0; i < 4; i++) y[i] = x[i] + lam * dx[i];
      if (y[0] > 0) {
        dens_jac(e, model, entropy, y, f, J, f32 ? Jf : nullptr, rmode);
        double gmax = 0.0;
        for (int i = 0; i < 4; i++) {
          const double r = fabs(f[i] - tgt[i]);
          gmax = (r > gmax || r != r) ? r : gmax;
        }
        if (gmax <= fres || h == 6) { have = true; break; }
      }
      lam *= 0.5;
    }
    if (!(y[0] > 0)) { y[0] = 0.5 * x[0]; have = false; }
    // progress test of the reference's solver (GSL hybrids, called from
    // src/rootfinder.cpp:206-416): the actual relative reduction of |F|^2;
    // five iterations below 0.1 or ten below 0.001 fail the attempt
    if (have) {
      double n0 = 0.0, n1 = 0.0;
      for (int i = 0; i < 4; i++) {
        n0 += F[i] * F[i];
        const double r = f[i] - tgt[i];
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
  *iters += max_it;
  return false;
}

__host__ __device__ inline double sgnd(double v) { return (0.0 < v) - (v < 0.0); }

// Seed sanitising and the perturbed-restart ladder of the reference
// (src/rootfinder.cpp:421-715).
__host__ __device__ inline bool find_root(const EosDev& e, int model, int entropy, const double* tgt, double* x,
                                          int* iters) {
  double lo[4], hi[4];
  model_box(e, model, lo, hi);
  double pos[4] = {x[0], x[1], x[2], x[3]};
  // the reduced modes start the frozen potentials at zero
  const int rmode = root_mode(e, model, tgt);
  for (int i = (rmode == 2 ? 1 : 2); rmode && i < 4; i++) pos[i] = 0.0;
  const double sg[4] = {1.0, sgnd(tgt[1]), sgnd(tgt[2]), sgnd(tgt[3])};
  for (int i = 0; i < 4; i++)
    if (pos[i] * pos[i] < 1e-10) pos[i] = fmin(0.5 * hi[i], 1.0) * sg[i];
  const double t0 = pos[0], b0 = pos[1], q0 = pos[2], s0 = pos[3];
  double seeds[10][4];
  const double tp = t0 + 0.2 * t0 > hi[0] ? hi[0] - 1 : t0 + 0.2 * t0;
  const double tm = t0 - 0.2 * t0 < lo[0] ? lo[0] + 1 : t0 - 0.2 * t0;
  const double bp = b0 + 0.2 * b0 > hi[1] ? hi[1] - 1 : b0 + 0.2 * b0;
  const double bm = b0 - 0.2 * b0 < lo[1] ? lo[1] + 1 : b0 - 0.2 * b0;
  const double sp = s0 + 0.2 * s0 > hi[3] ? hi[3] - 1 : s0 + 0.2 * s0;
  const double sm = s0 - 0.2 * s0 < lo[3] ? lo[3] + 1 : s0 - 0.2 * s0;
  const double qp = q0 + 0.2 * q0 > hi[2] ? hi[2] - 1 : q0 + 0.2 * q0;
  const double qm = q0 - 0.2 * q0 < lo[2] ? lo[2] + 1 : q0 - 0.2 * q0;
  auto clampT = [&](double v) { return (v < lo[0] || v > hi[0]) ? t0 : v; };
  const double list[10][4] = {{t0, b0, q0, s0},         {clampT(tp), b0, q0, s0}, {clampT(tm), b0, q0, s0},
                              {t0, bp, q0, s0},         {t0, bm, q0, s0},         {t0, b0, q0, sp},
                              {t0, b0, q0, sm},         {t0, b0, qp, s0},         {t0, b0, qm, s0},
                              {t0, fmin(0.5 * hi[1], 1.0) * sg[1], fmin(0.5 * hi[2], 1.0) * sg[2],
                               fmin(0.5 * hi[3], 1.0) * sg[3]}};
  (void)seeds;
  for (int a = 0; a < 10; a++) {
    double y[4] = {list[a][0], list[a][1], list[a][2], list[a][3]};
    if (newton_attempt(e, model, entropy, tgt, lo, hi, y, iters, 100, rmode)) {
      for (int i = 0; i < 4; i++) x[i] = y[i];
      return true;
    }
  }
  return false;
}

// Exact inverses of the conformal-diagonal model, the reference's last seed
// (include/eos_conformal_diagonal.h:49-76).
__host__ __device__ inline void confdiag_seed(const Scales& k, int entropy, const double* target, double* x) {
  const double den = 1.5874010519681994748 * cbrt(k.c);
  const double e0 = target[0], B = target[1], S = target[2], Q = target[3];
  if (entropy) {
    x[0] = cbrt(k.T0 * k.T0 * k.T0 * k.T0 * e0) / den;
  } else {
    const double ft = 4.0 / 3.0;
    const double disc = e0 - 3.0 * (pow(k.muB0 * fabs(B), ft) + pow(k.muS0 * fabs(S), ft) + pow(k.muQ0 * fabs(Q), ft)) /
                                 (4.0 * den);
    x[0] = k.T0 * pow(disc / (3.0 * k.c), 0.25);
  }
  x[1] = sgnd(B) * cbrt(k.muB0 * k.muB0 * k.muB0 * k.muB0 * fabs(B)) / den;
  x[2] = sgnd(Q) * cbrt(k.muQ0 * k.muQ0 * k.muQ0 * k.muQ0 * fabs(Q)) / den;
  x[3] = sgnd(S) * cbrt(k.muS0 * k.muS0 * k.muS0 * k.muS0 * fabs(S)) / den;
}

// Exact inverse of an analytic model in entropy mode, (s, B, Q, S) ->
// (T, muB, muQ, muS); false for the table.
//   conformal-diagonal: p = c T0^4 sum_k (X_k/X0_k)^4, so each density
//     d_k = 4 c T0^4 X_k^3 / X0_k^4 and X_k = cbrt(d_k X0_k^4 / (4 c T0^4));
//   conformal: p = c T0^4 x^2 with x = sum_k (X_k/X0_k)^2, so
//     d_k = 4 c T0^4 x X_k / X0_k^2; with a_k = X_k/X0_k and
//     d'_k = d_k X0_k / (4 c T0^4) = a_k x, x^3 = sum_k d'_k^2 and a_k = d'_k / x.
// Real cube root without an FP64 division: the FP32 estimate r0 of x^(-1/3)
// (rcbrtf of the rounded input, relative error d ~ 2^-23) refined by the
// third-order step of the binomial series r = r0 (1 - e)^(-1/3) =
// r0 (1 + e/3 + 2 e^2/9 + ...), e = 1 - x r0^3 (Householder's method of
// order 2 for x^(-1/3)); the truncation error, about 14 |e|^3 / 81 ~ 5 d^3,
// is far below FP64 precision, and cbrt(x) = x r^2 to a few ulp. Inputs
// outside the FP32 normal range go to cbrt.
__host__ __device__ inline double cbrt_refined(double x) {
  const double ax = fabs(x);
  if (ax == 0.0) return x;   // a zero density (no strangeness, say) is its own cube root
  if (!(ax > 1e-30 && ax < 1e30)) return cbrt(x);
  const double r0 = f64_of(rcbrtf(f32_rn(x)));
  const double e = fma(-(x * r0), r0 * r0, 1.0);
  const double r = fma(r0, e * fma(2.0 / 9.0, e, 1.0 / 3.0), r0);
  return x * (r * r);
}

__host__ __device__ inline bool analytic_seed(const EosDev& e, int model, const double* tgt, double* y) {
  if (model == M_TABLE || model == M_TANH) return false;
  const Scales k = model_scales(e, model);
  const double X0[4] = {k.T0, k.muB0, k.muQ0, k.muS0};
  const double ic4 = k.ic4;
  if (model == M_CDIAG) {
    for (int i = 0; i < 4; i++) {
      const double q = X0[i] * X0[i];
      y[i] = cbrt_refined(tgt[i] * q * q * ic4);
    }
    return y[0] > 0.0;
  }
  double d[4], x3 = 0.0;
  for (int i = 0; i < 4; i++) {
    d[i] = tgt[i] * X0[i] * ic4;
    x3 += d[i] * d[i];
  }
  const double xx = cbrt_refined(x3);
  if (!(xx > 0.0)) return false;
  const double ix = 1.0 / xx;
  for (int i = 0; i < 4; i++) y[i] = d[i] * ix * X0[i];
  return y[0] > 0.0;
}

// restrict_mu_T_ratios (src/eos.cpp:781-786): a table solution x = (T, muB,
// muQ, muS) with max |mu| > 3.5 T is refused.
__host__ __device__ inline bool mu_T_refused(const EosDev& e, int model, const double* x) {
  return e.restrict_mu_T && model == M_TABLE && fmax(fmax(fabs(x[1]), fabs(x[3])), fabs(x[2])) > 3.5 * x[0];
}

// (e|s, B, S, Q) -> (T, muB, muQ, muS) through the EoS chain with the
// reference's seeds (src/eos.cpp:629-804 entropy mode, :813-975 energy mode).
// seed_mode 1 (entropy mode) first tries Newton from the analytic model's
// exact inverse, seed_mode 2 from the given x (a learned seed) on the first
// model tried; then the reference's seeds. o_out, if given, receives the
// model thermodynamics at the solution (17 values). Returns the chain index
// used, or -1.
__host__ __device__ inline int eos_invert(const EosDev& e, int entropy, const double* target, int start, double* x,
                                          int* iters, int seed_mode = 0, double* o_out = nullptr) {
  const double tgt[4] = {target[0], target[1], target[3], target[2]};  // (e|s, B, Q, S)
  const int n = chain_len(e.kind);
  const Scales cdk = model_scales(e, M_CDIAG);
  const double prev[4] = {x[0], x[1], x[2], x[3]};
  int it = 0;
  for (int k = entropy ? (start > 0 ? start : 0) : 0; k < n; k++) {
    const int model = chain_model(e.kind, k);
    double y[4];
    bool ok = false;
    if (seed_mode == 2 && k == (entropy ? (start > 0 ? start : 0) : 0)) {
      // learned seed (the given x) for the first model tried
      double lo[4], hi[4];
      model_box(e, model, lo, hi);
      for (int i = 0; i < 4; i++) y[i] = fmin(fmax(prev[i], lo[i]), hi[i]);
      ok = y[0] > 0.0 && newton_attempt(e, model, entropy, tgt, lo, hi, y, &it, 100, root_mode(e, model, tgt));
      if (ok) {   // a root the c_s^2 guard rejects leaves this model to the reference seeds
        double o[17];
        model_thermo(e, model, y, o);
        ok = o[6] >= 0.0 && o[6] <= 1.0;
        if (!ok)
          for (int i = 0; i < 4; i++) y[i] = prev[i];
      }
    } else if (entropy && seed_mode == 1 && analytic_seed(e, model, tgt, y)) {
      // the exact inverse is accepted when it meets the reference's residual
      // test (max |F| < 1e-10); otherwise Newton starts from it
      double o[17];
      model_thermo(e, model, y, o);
      const double fres = fmax(fmax(fabs(o[1] - tgt[0]), fabs(o[2] - tgt[1])),
                               fmax(fabs(o[4] - tgt[2]), fabs(o[3] - tgt[3])));
      if (fres < 1e-10 && o[6] >= 0.0 && o[6] <= 1.0) {
        for (int i = 0; i < 4; i++) x[i] = y[i];
        if (o_out)
          for (int i = 0; i < 17; i++) o_out[i] = o[i];
        *iters = it;
        return k;
      }
      double lo[4], hi[4];
      model_box(e, model, lo, hi);
      ok = newton_attempt(e, model, 1, tgt, lo, hi, y, &it);
    }
    if (ok) {
    } else if (entropy) {
      for (int i = 0; i < 4; i++) y[i] = prev[i];
      ok = find_root(e, model, 1, tgt, y, &it);
      if (!ok) { y[0] = prev[0]; y[1] = y[2] = y[3] = 0.0; ok = find_root(e, model, 1, tgt, y, &it); }
      if (!ok) {
        y[0] = 580.0 / kHbarcMeVfm; y[1] = sgnd(tgt[1]); y[2] = sgnd(tgt[2]); y[3] = sgnd(tgt[3]);
        ok = find_root(e, model, 1, tgt, y, &it);
      }
      if (!ok) { confdiag_seed(cdk, 1, target, y); ok = find_root(e, model, 1, tgt, y, &it); }
    } else {
      y[0] = 580.0 / kHbarcMeVfm; y[1] = sgnd(tgt[1]); y[2] = sgnd(tgt[2]); y[3] = sgnd(tgt[3]);
      ok = find_root(e, model, 0, tgt, y, &it);
      if (!ok) { confdiag_seed(cdk, 0, target, y); ok = find_root(e, model, 0, tgt, y, &it); }
    }
    // a solution is a finite point with T > 0
    ok = ok && y[0] > 0.0 && y[0] <= 1e300 && fabs(y[1]) <= 1e300 && fabs(y[2]) <= 1e300 && fabs(y[3]) <= 1e300;
    if (ok) {
      double o[17];
      model_thermo(e, model, y, o);
      if (!(o[6] >= 0.0 && o[6] <= 1.0)) continue;   // prohibit unstable / acausal cs2
      if (mu_T_refused(e, model, y)) continue;
      for (int i = 0; i < 4; i++) x[i] = y[i];
      if (o_out)
        for (int i = 0; i < 17; i++) o_out[i] = o[i];
      *iters = it;
      return k;
    }
  }
  *iters = it;
  return -1;
}

// The first attempt of eos_invert (first model of the chain, its first seed)
// with Newton capped at max_it iterations. Returns the chain index, with the
// same x, iterations and o_out as eos_invert gives whenever that attempt
// succeeds, or -2 when it does not settle the row (the caller then runs
// eos_invert from the same seed). Not for seed_mode 1.
__host__ __device__ inline int eos_invert_first(const EosDev& e, int entropy, const double* target, int start,
                                                double* x, int* iters, int seed_mode, int max_it, double* o_out) {
  const double tgt[4] = {target[0], target[1], target[3], target[2]};  // (e|s, B, Q, S)
  const int k = entropy ? (start > 0 ? start : 0) : 0;
  if (k >= chain_len(e.kind) || seed_mode == 1) return -2;
  const int model = chain_model(e.kind, k);
  double lo[4], hi[4];
  model_box(e, model, lo, hi);
  double y[4];
  const int rmode = root_mode(e, model, tgt);
  if (seed_mode == 2) {
    for (int i = 0; i < 4; i++) y[i] = fmin(fmax(x[i], lo[i]), hi[i]);
    if (!(y[0] > 0.0)) return -2;
  } else {
    if (entropy) {
      for (int i = 0; i < 4; i++) y[i] = x[i];
    } else {
      y[0] = 580.0 / kHbarcMeVfm; y[1] = sgnd(tgt[1]); y[2] = sgnd(tgt[2]); y[3] = sgnd(tgt[3]);
    }
    // find_root's seed sanitising (and its zeroing of frozen potentials)
    for (int i = (rmode == 2 ? 1 : 2); rmode && i < 4; i++) y[i] = 0.0;
    const double sg[4] = {1.0, sgnd(tgt[1]), sgnd(tgt[2]), sgnd(tgt[3])};
    for (int i = 0; i < 4; i++)
      if (y[i] * y[i] < 1e-10) y[i] = fmin(0.5 * hi[i], 1.0) * sg[i];
  }
  int it = 0;
  if (!newton_attempt(e, model, entropy, tgt, lo, hi, y, &it, max_it, rmode)) return -2;
  if (!(y[0] > 0.0 && y[0] <= 1e300 && fabs(y[1]) <= 1e300 && fabs(y[2]) <= 1e300 && fabs(y[3]) <= 1e300))
    return -2;
  double o[17];
  model_thermo(e, model, y, o);
  if (!(o[6] >= 0.0 && o[6] <= 1.0) || mu_T_refused(e, model, y)) return -2;
  for (int i = 0; i < 4; i++) x[i] = y[i];
  if (o_out)
    for (int i = 0; i < 17; i++) o_out[i] = o[i];
  *iters = it;
  return k;
}

// The first attempt of eos_invert in seed mode 1 (entropy mode) when the
// analytic inverse settles it: the model tried first is conformal or
// conformal-diagonal and its exact inverse passes the residual and c_s^2
// tests. Returns the chain index with x and o_out as eos_invert gives them
// then (no Newton steps), or -2 (the caller runs eos_invert). Only the two
// analytic models are compiled in, so a kernel built on it stays small.
__host__ __device__ inline int eos_analytic_first(const EosDev& e, const double* target, int start, double* x,
                                                  double* o_out) {
  const double tgt[4] = {target[0], target[1], target[3], target[2]};  // (s, B, Q, S)
  const int k = start > 0 ? start : 0;
  if (k >= chain_len(e.kind)) return -2;
  const int model = chain_model(e.kind, k);
  if (model != M_CONF && model != M_CDIAG) return -2;
  double y[4];
  if (!analytic_seed(e, model, tgt, y)) return -2;
  const Scales sc = model_scales(e, model);
  double o[17];
  if (model == M_CONF) conformal_thermo(sc, y, o);
  else confdiag_thermo(sc, y, o);
  const double fres = fmax(fmax(fabs(o[1] - tgt[0]), fabs(o[2] - tgt[1])),
                           fmax(fabs(o[4] - tgt[2]), fabs(o[3] - tgt[3])));
  if (!(fres < 1e-10 && o[6] >= 0.0 && o[6] <= 1.0)) return -2;
  for (int i = 0; i < 4; i++) x[i] = y[i];
  for (int i = 0; i < 17; i++) o_out[i] = o[i];
  return k;
}

// a^T m^-1 b with the reference's guard on m11, m22 (src/eos_derivatives.cpp:457-560).
__host__ __device__ inline double aTmb(const double* a, double m[3][3], const double* b) {
  const double EPS = 1e-3;
  if (fabs(m[1][1]) < EPS) m[1][1] = (m[1][1] >= 0.0 ? EPS : -EPS);
  if (fabs(m[2][2]) < EPS) m[2][2] = (m[2][2] >= 0.0 ? EPS : -EPS);
  double y[3] = {b[0], b[1], b[2]};
  for (int k = 0; k < 3; k++) {
    int p = k;
    for (int i = k + 1; i < 3; i++) if (fabs(m[i][k]) > fabs(m[p][k])) p = i;
    if (p != k) {
      for (int j = 0; j < 3; j++) { double t = m[k][j]; m[k][j] = m[p][j]; m[p][j] = t; }
      double t = y[k]; y[k] = y[p]; y[p] = t;
    }
    for (int i = k + 1; i < 3; i++) {
      const double f = m[i][k] / m[k][k];
      for (int j = k; j < 3; j++) m[i][j] -= f * m[k][j];
      y[i] -= f * y[k];
    }
  }
  double z[3];
  for (int k = 2; k >= 0; k--) {
    double acc = y[k];
    for (int j = k + 1; j < 3; j++) acc -= m[k][j] * z[j];
    z[k] = acc / m[k][k];
  }
  return a[0] * z[0] + a[1] * z[1] + a[2] * z[2];
}

struct Chi { double t2, tb, tq, ts, b2, q2, s2, bq, bs, sq; };

// Schur-complement terms of the reference (src/eos_derivatives.cpp:33-455).
// which: 0 term1; 1..3 term2(B,S,Q); 4..6 term3(B,S,Q); 7 + 3*j + i term4(j,i).
// rm: the reduced modes (2 T-only, 1 baryon-only; src/eos_derivatives.cpp:
// 33-45, :74-90, :160-172, :240-254): the Schur complements over the active
// rows only, with the reference's 1e-30 guards. which: 0 term1, 1..3
// term2(B, S, Q), 4..6 term3(B, S, Q), 7 + 3j + i term4(j, i).
__host__ __device__ inline double schur_term(const Chi& x, int which, int rm = 0) {
  if (rm == 2) return which == 0 ? x.t2 : 0.0;
  if (rm == 1) {
    if (which == 0) return x.t2 - (x.tb * x.tb) / (x.b2 + 1e-30);
    if (which == 1) return x.tb - (x.t2 * x.b2) / (x.tb + 1e-30);
    if (which == 4) return x.tb - (x.b2 * x.t2) / (x.tb + 1e-30);
    if (which == 7) return x.b2 - (x.tb * x.tb) / (x.t2 + 1e-30);
    return 0.0;
  }
  double a[3], b[3], m[3][3], base;
#define SET3(v, p, q, r) { v[0] = (p); v[1] = (q); v[2] = (r); }
#define SETM(a0, a1, a2, b0, b1, b2, c0, c1, c2) \
  { m[0][0] = a0; m[0][1] = a1; m[0][2] = a2; m[1][0] = b0; m[1][1] = b1; m[1][2] = b2; m[2][0] = c0; m[2][1] = c1; m[2][2] = c2; }
  switch (which) {
    case 0: SET3(a, x.tb, x.ts, x.tq); SET3(b, x.tb, x.ts, x.tq);
      SETM(x.b2, x.bs, x.bq, x.bs, x.s2, x.sq, x.bq, x.sq, x.q2); base = x.t2; break;
    case 1: SET3(a, x.t2, x.ts, x.tq); SET3(b, x.b2, x.bs, x.bq);
      SETM(x.tb, x.bs, x.bq, x.ts, x.s2, x.sq, x.tq, x.sq, x.q2); base = x.tb; break;
    case 2: SET3(a, x.t2, x.tb, x.tq); SET3(b, x.bs, x.s2, x.sq);
      SETM(x.tb, x.b2, x.bq, x.ts, x.bs, x.sq, x.tq, x.bq, x.q2); base = x.ts; break;
    case 3: SET3(a, x.t2, x.tb, x.ts); SET3(b, x.bq, x.sq, x.q2);
      SETM(x.tb, x.b2, x.bs, x.ts, x.bs, x.s2, x.tq, x.bq, x.sq); base = x.tq; break;
    case 4: SET3(a, x.b2, x.bs, x.bq); SET3(b, x.t2, x.ts, x.tq);
      SETM(x.tb, x.ts, x.tq, x.bs, x.s2, x.sq, x.bq, x.sq, x.q2); base = x.tb; break;
    case 5: SET3(a, x.bs, x.s2, x.sq); SET3(b, x.t2, x.tb, x.tq);
      SETM(x.tb, x.ts, x.tq, x.b2, x.bs, x.bq, x.bq, x.sq, x.q2); base = x.ts; break;
    case 6: SET3(a, x.bq, x.sq, x.q2); SET3(b, x.t2, x.tb, x.ts);
      SETM(x.tb, x.ts, x.tq, x.b2, x.bs, x.bq, x.bs, x.s2, x.sq); base = x.tq; break;
    // term4(j, i), j: charge of the density, i: charge of the potential (0 B, 1 S, 2 Q)
    case 7 + 0 * 3 + 0: SET3(a, x.tb, x.bs, x.bq); SET3(b, x.tb, x.bs, x.bq);
      SETM(x.t2, x.ts, x.tq, x.ts, x.s2, x.sq, x.tq, x.sq, x.q2); base = x.b2; break;
    case 7 + 1 * 3 + 0: SET3(a, x.ts, x.s2, x.sq); SET3(b, x.tb, x.b2, x.bq);
      SETM(x.t2, x.ts, x.tq, x.tb, x.bs, x.bq, x.tq, x.sq, x.q2); base = x.bs; break;
    case 7 + 2 * 3 + 0: SET3(a, x.tq, x.sq, x.q2); SET3(b, x.tb, x.b2, x.bs);
      SETM(x.t2, x.ts, x.tq, x.tb, x.bs, x.bq, x.ts, x.s2, x.sq); base = x.bq; break;
    case 7 + 0 * 3 + 1: SET3(a, x.tb, x.b2, x.bq); SET3(b, x.ts, x.s2, x.sq);
      SETM(x.t2, x.tb, x.tq, x.ts, x.bs, x.sq, x.tq, x.bq, x.q2); base = x.bs; break;
    case 7 + 1 * 3 + 1: SET3(a, x.ts, x.bs, x.sq); SET3(b, x.ts, x.bs, x.sq);
      SETM(x.t2, x.tb, x.tq, x.tb, x.b2, x.bq, x.tq, x.bq, x.q2); base = x.s2; break;
    case 7 + 2 * 3 + 1: SET3(a, x.tq, x.bq, x.q2); SET3(b, x.ts, x.bs, x.s2);
      SETM(x.t2, x.tb, x.tq, x.tb, x.b2, x.bq, x.ts, x.bs, x.sq); base = x.sq; break;
    case 7 + 0 * 3 + 2: SET3(a, x.tb, x.b2, x.bs); SET3(b, x.tq, x.sq, x.q2);
      SETM(x.t2, x.tb, x.ts, x.ts, x.bs, x.s2, x.tq, x.bq, x.sq); base = x.bq; break;
    case 7 + 1 * 3 + 2: SET3(a, x.ts, x.bs, x.s2); SET3(b, x.tq, x.bq, x.q2);
      SETM(x.t2, x.tb, x.ts, x.tb, x.b2, x.bs, x.tq, x.bq, x.sq); base = x.sq; break;
    default: SET3(a, x.tq, x.bq, x.sq); SET3(b, x.tq, x.bq, x.sq);
      SETM(x.t2, x.tb, x.ts, x.tb, x.b2, x.bs, x.ts, x.bs, x.s2); base = x.q2; break;
  }
#undef SET3
#undef SETM
  return base - aTmb(a, m, b);
}

// Derived thermodynamics at a solution: T mu p s rho e w cs2 and dw/ds, dw/drho
// (reference include/eos.h:121-175, src/eos.cpp:276-344). th must hold NTH doubles.
// o: the model thermodynamics at x (model_thermo of the chain's model k).
// fp32_derivs: the conformal-diagonal enthalpy derivatives dw/ds, dw/drho in
// FP32 arithmetic (they feed only FP32 equations of motion in the mixed form).
// G = H^-1 over the rows keep[0..m) (Gauss-Jordan, partial pivoting) in the
// arithmetic R; zero elsewhere.
template <class R>
__host__ __device__ inline void hessian_inverse(const double H[4][4], const int* keep, int m, double G[4][4]) {
  R A[4][8];
  for (int i = 0; i < 4; i++) for (int j = 0; j < 8; j++) A[i][j] = R(0);
  for (int i = 0; i < m; i++) {
    for (int j = 0; j < m; j++) A[i][j] = R(H[keep[i]][keep[j]]);
    A[i][m + i] = R(1);
  }
  for (int col = 0; col < m; col++) {
    int p = col;
    for (int r = col + 1; r < m; r++) if (fabs(A[r][col]) > fabs(A[p][col])) p = r;
    if (p != col) for (int j = 0; j < 2 * m; j++) { R t = A[col][j]; A[col][j] = A[p][j]; A[p][j] = t; }
    const R ipiv = R(1) / A[col][col];
    for (int j = 0; j < 2 * m; j++) A[col][j] *= ipiv;
    for (int r = 0; r < m; r++) {
      if (r == col || A[r][col] == R(0)) continue;
      const R f = A[r][col];
      for (int j = 0; j < 2 * m; j++) A[r][j] -= f * A[col][j];
    }
  }
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) G[i][j] = 0.0;
  for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) G[keep[i]][keep[j]] = double(A[i][m + j]);
}

__host__ __device__ inline void set_thermo_o(const EosDev& e, int k, const double* x, const double* o, double* th,
                                             bool fp32_derivs = false) {
  const int model = chain_model(e.kind, k);
  const int rm = frozen_mode(e, model);
  const double T = x[0], mB = x[1], mQ = x[2], mS = x[3];
  const double s = o[1], B = o[2], S = o[3], Q = o[4];
  th[T_T] = T; th[T_MUB] = mB; th[T_MUS] = mS; th[T_MUQ] = mQ;
  th[T_P] = o[0]; th[T_S] = s; th[T_RB] = B; th[T_RS] = S; th[T_RQ] = Q; th[T_E] = o[5];
  th[T_W] = o[5] + o[0]; th[T_CS2] = o[6];
  const Chi X{o[16], o[13], o[14], o[15], o[7], o[8], o[9], o[10], o[11], o[12]};
  const bool hB = fabs(B) > kTiny, hS = fabs(S) > kTiny, hQ = fabs(Q) > kTiny;
  if (e.thermo_mode == 1) {
    // exact: G = H^-1 over the Hessian rows that are not identically zero
    double H[4][4] = {{X.t2, X.tb, X.ts, X.tq}, {X.tb, X.b2, X.bs, X.bq}, {X.ts, X.bs, X.s2, X.sq},
                      {X.tq, X.bq, X.sq, X.q2}};
    const double rho[4] = {0.0, B, S, Q};
    const bool act[4] = {true, hB, hS, hQ};
    const double mu[4] = {T, mB, mS, mQ};
    if (model == M_CDIAG) {
      // diagonal Hessian: G = diag(1/H_aa) over the non-zero rows (the
      // elimination below gives the same reciprocals)
      for (int a = 0; a < 4; a++) {
        const double Haa = H[a][a];
        if (fp32_derivs) {
          const float G = Haa != 0.0 ? 1.0f / f32_rn(Haa) : 0.0f;
          th[T_DWDS + a] = (a == 0 || act[a]) ? f64_of(f32_rn(mu[a]) + f32_rn(a == 0 ? s : rho[a]) * G) : mu[a];
        } else {
          const double G = Haa != 0.0 ? 1.0 / Haa : 0.0;
          th[T_DWDS + a] = (a == 0 || act[a]) ? mu[a] + (a == 0 ? s : rho[a]) * G : mu[a];
        }
      }
      return;
    }
    int keep[4], m = 0;
    for (int i = 0; i < 4; i++) {
      bool zero = true;
      for (int j = 0; j < 4; j++) zero = zero && (H[i][j] == 0.0);
      if (!zero) keep[m++] = i;
    }
    double G[4][4];
    if (fp32_derivs) hessian_inverse<float>(H, keep, m, G);
    else hessian_inverse<double>(H, keep, m, G);
    for (int a = 0; a < 4; a++) {
      double acc = mu[a];
      if (a == 0 || act[a]) {
        acc += s * G[0][a];
        for (int b = 1; b < 4; b++) if (act[b]) acc += rho[b] * G[b][a];
      }
      th[T_DWDS + a] = acc;
    }
    return;
  }
  double ct = 0.0;
  if (hB) ct += B / schur_term(X, 1, rm);
  if (hQ) ct += Q / schur_term(X, 3, rm);
  if (hS) ct += S / schur_term(X, 2, rm);
  th[T_DWDS] = T + s / schur_term(X, 0, rm) + ct;
  ct = 0.0;
  if (hB) {
    ct += s / schur_term(X, 4, rm) + B / schur_term(X, 7 + 0, rm);
    if (hQ) ct += Q / schur_term(X, 7 + 0 * 3 + 2, rm);
    if (hS) ct += S / schur_term(X, 7 + 0 * 3 + 1, rm);
  }
  th[T_DWDB] = mB + ct;
  ct = 0.0;
  if (hS) {
    ct += s / schur_term(X, 5, rm) + S / schur_term(X, 7 + 1 * 3 + 1, rm);
    if (hB) ct += B / schur_term(X, 7 + 1 * 3 + 0, rm);
    if (hQ) ct += Q / schur_term(X, 7 + 1 * 3 + 2, rm);
  }
  th[T_DWDSS] = mS + ct;
  ct = 0.0;
  if (hQ) {
    ct += s / schur_term(X, 6, rm) + Q / schur_term(X, 7 + 2 * 3 + 2, rm);
    if (hB) ct += B / schur_term(X, 7 + 2 * 3 + 0, rm);
    if (hS) ct += S / schur_term(X, 7 + 2 * 3 + 1, rm);
  }
  th[T_DWDQ] = mQ + ct;
}

// The twelve derivatives of alpha_a = mu_a / T at fixed (s, rho) read by the
// diffusion sector (src/eos.cpp:337-493, dalpha_Bds .. dalpha_QdQ), at a
// solution x with model thermodynamics o. out[a] = dalpha_a/ds,
// out[3 + 3a + b] = dalpha_a/drho_b, a, b over (B, S, Q). The reference
// chain (thermo_mode 0): dalpha_a/ds = -mu_a/T^2 / term1 + [rho_a] (1/T) /
// term2(a); dalpha_a/drho_b = [rho_b] (-mu_a/T^2 / term3(b) + [rho_a] (1/T) /
// term4(b, a)), [rho] meaning |rho| > TINY, dalpha_BdB with its 1/T term
// first. thermo_mode 1: the same with the entries of H^-1 for 1/term.
__host__ __device__ inline void alpha_derivs_o(const EosDev& e, int k, const double* x, const double* o,
                                               double* out) {
  const int rm = frozen_mode(e, chain_model(e.kind, k));
  const double T = x[0];
  const double mu[3] = {x[1], x[3], x[2]};
  const double rho[3] = {o[2], o[3], o[4]};
  const Chi X{o[16], o[13], o[14], o[15], o[7], o[8], o[9], o[10], o[11], o[12]};
  bool h[3];
  for (int a = 0; a < 3; a++) h[a] = fabs(rho[a]) > kTiny;
  const double iT = 1 / T;
  if (e.thermo_mode == 1) {
    const int model = chain_model(e.kind, k);
    double H[4][4] = {{X.t2, X.tb, X.ts, X.tq}, {X.tb, X.b2, X.bs, X.bq}, {X.ts, X.bs, X.s2, X.sq},
                      {X.tq, X.bq, X.sq, X.q2}};
    if (model == M_CDIAG)
      for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) if (i != j) H[i][j] = 0.0;
    int keep[4], m = 0;
    for (int i = 0; i < 4; i++) {
      bool zero = true;
      for (int j = 0; j < 4; j++) zero = zero && (H[i][j] == 0.0);
      if (!zero) keep[m++] = i;
    }
    double G[4][4];
    hessian_inverse<double>(H, keep, m, G);
    for (int a = 0; a < 3; a++) {
      double ct = 0.0;
      if (h[a]) ct += iT * G[a + 1][0];
      out[a] = -mu[a] / T / T * G[0][0] + ct;
      for (int b = 0; b < 3; b++) {
        double v = 0.0;
        if (h[b]) {
          v += -mu[a] / T / T * G[0][b + 1];
          if (h[a]) v += iT * G[a + 1][b + 1];
        }
        out[3 + 3 * a + b] = v;
      }
    }
    return;
  }
  const double t1 = schur_term(X, 0, rm);
  for (int a = 0; a < 3; a++) {
    double ct = 0.0;
    if (h[a]) ct += iT / schur_term(X, 1 + a, rm);
    out[a] = -mu[a] / T / T / t1 + ct;
  }
  for (int b = 0; b < 3; b++) {
    if (!h[b]) {
      for (int a = 0; a < 3; a++) out[3 + 3 * a + b] = 0.0;
      continue;
    }
    const double t3 = schur_term(X, 4 + b, rm);
    for (int a = 0; a < 3; a++) {
      double v = 0.0;
      if (a == 0 && b == 0) {
        v += iT / schur_term(X, 7, rm) - mu[0] / T / T / t3;
      } else {
        v += -mu[a] / T / T / t3;
        if (h[a]) v += iT / schur_term(X, 7 + 3 * b + a, rm);
      }
      out[3 + 3 * a + b] = v;
    }
  }
}

#ifdef __CUDACC__
// EoS_Interpolator::fill_thermodynamics and interpolate4D
// (src/eos_interpolator.cpp:531-739) for one point: densities clamped to
// max(0.001, |x|) (the tables hold positive densities only, and the
// chemical potentials are returned as tabulated), the tile of each axis by
// its decade (the count of tile edges 10^(e_lo + j) at or below x, clamped to
// the tiles present), the cell by floor((x - min) / step) clamped to the tile,
// and the 16-corner multilinear sum in the reference's corner order (bit i of
// the corner number is axis i) with every rounding explicit. out[11] in
// kPreVars order.
__device__ inline void preinv_lookup(const PreinvView& P, const double* sBSQ, double* out) {
  double pos[4];
  pos[0] = fmax(0.001, sBSQ[0]);
  for (int k = 1; k < 4; k++) pos[k] = fmax(0.001, fabs(sBSQ[k]));
  int t[4], idx[4];
  double x[4];
  for (int k = 0; k < 4; k++) {
    int tk = 0;
    for (int j = 1; j < P.nt[k]; j++) tk += (pos[k] >= P.mn[k][j]) ? 1 : 0;
    t[k] = tk;
    const double mn = P.mn[k][tk], st = P.st[k][tk];
    int ik = (int)floor(__ddiv_rn(__dsub_rn(pos[k], mn), st));
    ik = ik < 0 ? 0 : ik;
    // the +1 corner stays inside the tile (the reference clamps to N - 1)
    ik = ik > P.N - 2 ? P.N - 2 : ik;
    idx[k] = ik;
    x[k] = __ddiv_rn(__dsub_rn(__dsub_rn(pos[k], mn), __dmul_rn((double)ik, st)), st);
  }
  const long tile = (((long)t[0] * P.nt[1] + t[1]) * P.nt[2] + t[2]) * P.nt[3] + t[3];
  const long N = P.N, tn = N * N * N * N;
  const double* base = P.v + (size_t)tile * tn * kPreVars;
  double phi[16];
  for (int c = 0; c < 16; c++) {
    double ph = 1.0;
    for (int i = 0; i < 4; i++) ph = __dmul_rn(ph, ((c >> i) & 1) ? x[i] : __dsub_rn(1.0, x[i]));
    phi[c] = ph;
  }
  for (int v = 0; v < kPreVars; v++) out[v] = 0.0;
  for (int c = 0; c < 16; c++) {
    const long node = (((long)(idx[0] + (c & 1)) * N + idx[1] + ((c >> 1) & 1)) * N + idx[2] + ((c >> 2) & 1)) * N +
                      idx[3] + ((c >> 3) & 1);
    const double* nv = base + (size_t)node * kPreVars;
    for (int v = 0; v < kPreVars; v++) out[v] = __dadd_rn(out[v], __dmul_rn(phi[c], nv[v]));
  }
}
#endif

__host__ __device__ inline void set_thermo(const EosDev& e, int k, const double* x, double* th) {
  double o[17];
  model_thermo(e, chain_model(e.kind, k), x, o);
  set_thermo_o(e, k, x, o, th);
}

}  // namespace ccake
