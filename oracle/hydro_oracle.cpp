// CPU oracle: transport coefficients, shear-tensor constraints, the MRF
// equations of motion (ideal + shear + bulk + diffusion, Milne and Cartesian
// coordinates), the midpoint RK2 evolver, conservation sums, initialisation
// and the freeze-out stage.
// TEST INFRASTRUCTURE ONLY (see oracle.hpp).
#include "oracle.hpp"
#include "table_oracle.hpp"

#include <algorithm>
#include <cmath>

namespace orc {

namespace {

// Milne index helpers (include/milne.hpp). Vector<D>::make_covariant flips the
// sign of every component and, except in 2-D, multiplies the last one by t^2
// (:92-96, 2-D specialisation :354); make_contravariant is the inverse (:103-107).
inline void cov_D(int D, double* v, double t2) {
  if (D == 2) { v[0] = -v[0]; v[1] = -v[1]; return; }
  for (int i = 0; i < D - 1; i++) v[i] = -v[i];
  v[D - 1] *= -t2;
}
inline void contra_D(int D, double* v, double t2) {
  if (D == 2) { v[0] = -v[0]; v[1] = -v[1]; return; }
  for (int i = 0; i < D - 1; i++) v[i] = -v[i];
  v[D - 1] *= -1. / t2;
}
// delta_i_eta<D> (:1095-1110). In 2-D the reference also reads index 2 of a
// two-element vector (out of bounds); that read is taken as zero here.
inline double dEta(int D, int i) { return (D == 3 && i == 2) ? 1.0 : 0.0; }

struct Coefs {
  double eta, tau_pi, zeta, tau_Pi, delta_PiPi, delta_pipi, lambda_piPi, lambda_Pipi, phi1, phi3,
      phi6, phi7, tau_pipi;
};

// src/transport_coefficients.cpp:620-900
double eta_of(const Config& c, double T, double w) {
  if (T <= 0.0) return 0.0;
  return c.eta_over_s * (w / T);
}
double tau_pi_of(const Config& c, double eta, double w) {
  if (c.shear_relax_mode == kTauPiGubser) return (5.0 * eta) / w;
  if (c.shear_relax_mode == kTauPiMinval) return std::max((5.0 * eta) / w, 0.001);
  return std::max(5.0 * eta / w, 0.005);
}
double zeta_of(const Config& c, double T, double w, double cs2) {
  switch (c.zeta_mode) {
    case kZetaConstant: return c.zeta_over_s * (w / T);
    case kZetaCs2: {
      double factor = 1.0;
      if (c.modulate_zeta_with_tanh) {
        const double Ttr = 150.0 / kHbarcMeVfm, Tsc = 10.0 / kHbarcMeVfm;
        double th = std::tanh((T - Ttr) / Tsc), xp = std::pow(T / Ttr, c.zeta_cs2_p);
        factor = 0.5 * (1.0 + xp) + 0.5 * (1.0 - xp) * th;
      }
      double zs = c.zeta_cs2_A * factor * std::pow((1.0 / 3.0) - std::min(cs2, 1.0), c.zeta_cs2_p);
      return zs * w / T;
    }
    case kZetaPeaked: {
      // zeta/s peaked at T = zeta_peak_T (Gaussian of width zeta_peak_width),
      // height zeta_over_s: the bulk mode requested for the 3+1-D run.
      double x = (T - c.zeta_peak_T) / c.zeta_peak_width;
      return c.zeta_over_s * std::exp(-0.5 * x * x) * (w / T);
    }
    default: return 0.005 * (w / T);
  }
}
double tau_Pi_of(const Config& c, double zeta, double w, double cs2) {
  const double p = c.zeta_cs2_p;
  const double cc = cs2 > 1 ? 1 : cs2;
  if (std::pow((1.0 / 3.0 - cc), p) < 1e-10) return 1e10;
  return std::max(5.0 * zeta / (std::pow((1.0 / 3.0 - cc), p) * w), 0.1);
}

Coefs coefs(const Config& c, const double* th) {
  Coefs k;
  const double T = th[kT], w = th[kW], cs2 = th[kCs2], p = th[kP];
  k.eta = eta_of(c, T, w);
  k.tau_pi = tau_pi_of(c, k.eta, w);
  k.zeta = zeta_of(c, T, w, cs2);
  k.tau_Pi = tau_Pi_of(c, k.zeta, w, cs2);
  // second-order coefficients by mode (src/transport_coefficients.cpp:
  // 380-560 switches, :704-912 the functions): 0 DEFAULT, 1 IS, 2 disabled
  auto pick = [](int32_t mode, double def, double is) { return mode == 2 ? 0.0 : (mode == 1 ? is : def); };
  k.delta_PiPi = pick(c.delta_PiPi_mode, 2. * k.tau_Pi / 3.0, k.tau_Pi);
  k.delta_pipi = pick(c.delta_pipi_mode, 4. * k.tau_pi / 3.0, k.tau_pi);
  k.lambda_piPi = pick(c.lambda_piPi_mode, 6. / 5. * k.tau_pi, 0.0);
  const double cc = cs2 > 1 ? 1 : cs2;
  k.lambda_Pipi = pick(c.lambda_Pipi_mode, 8. * (1. / 3. - cc) * k.tau_Pi / 5., 0.0);
  k.phi1 = 0.0;
  k.phi3 = 0.0;
  k.phi6 = 0.0;
  k.phi7 = pick(c.phi7_mode, 9. / (70. * p), 0.0);
  k.tau_pipi = pick(c.tau_pipi_mode, 10. * k.tau_pi / 7.0, 0.0);
  return k;
}

inline double gamma_of(int D, const double* u, double t2) {
  double uc[3] = {u[0], u[1], u[2]};
  cov_D(D, uc, t2);
  double c = 0;
  for (int i = 0; i < D; i++) c += uc[i] * u[i];
  return std::sqrt(1 - c);
}

// inverse of a D x D matrix by cofactors (include/milne.hpp:788-834)
void inverse(int D, const double* A, double* Ai) {
  if (D == 1) { Ai[0] = 1. / A[0]; return; }
  if (D == 2) {
    double det = A[0] * A[3] - A[1] * A[2];
    Ai[0] = A[3] / det; Ai[1] = -A[1] / det; Ai[2] = -A[2] / det; Ai[3] = A[0] / det;
    return;
  }
#define M(i, j) A[(i) * 3 + (j)]
  double det = M(0, 0) * M(1, 1) * M(2, 2) + M(0, 1) * M(1, 2) * M(2, 0) + M(0, 2) * M(1, 0) * M(2, 1) -
               M(0, 2) * M(1, 1) * M(2, 0) - M(0, 1) * M(1, 0) * M(2, 2) - M(0, 0) * M(1, 2) * M(2, 1);
  Ai[0] = (M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1)) / det;
  Ai[1] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) / det;
  Ai[2] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) / det;
  Ai[3] = (M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2)) / det;
  Ai[4] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) / det;
  Ai[5] = (M(0, 2) * M(1, 0) - M(0, 0) * M(1, 2)) / det;
  Ai[6] = (M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0)) / det;
  Ai[7] = (M(0, 1) * M(2, 0) - M(0, 0) * M(2, 1)) / det;
  Ai[8] = (M(0, 0) * M(1, 1) - M(0, 1) * M(1, 0)) / det;
#undef M
}

// Diffusion coefficients, src/transport_coefficients.cpp:571-617 (kappa,
// tauq), :918-973 (default_kappa = kappa/T^2 T^2, default_tauq = 0.2/T on
// the diagonal), :981-1040 (kappaB_coth, tauqB_only) and :1048-1057 (the
// Gaussian suppression near the critical point, table EoS only). tq, kq are
// row-major 3x3 over (B, S, Q).
void diffusion_coefs(const Config& c, const double* th, bool table_eos, double* tq, double* kq) {
  const double T = th[kT];
  for (int k = 0; k < 9; k++) tq[k] = kq[k] = 0.0;
  if (c.diffusion_mode == 2) {
    const double muB = th[kMuB], nB = th[kRhoB], w = th[kW];
    const double x = (T > kTiny) ? muB / T : 0.0;
    if (T > kTiny && std::fabs(w) > kTiny && std::fabs(x) > 1.0e-2) {
      const double kB = (c.C_B / T) * nB * ((1.0 / 3.0) / std::tanh(x) - nB * T / w);
      if (std::isfinite(kB) && kB > 0.0) kq[0] = kB;
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
    const double dT = T - c.crit_T / kHbarcMeVfm, dm = th[kMuB] - c.crit_muB / kHbarcMeVfm;
    const double sT = c.crit_wT / kHbarcMeVfm, sm = c.crit_wmuB / kHbarcMeVfm;
    const double ex = 0.5 * (dT * dT / (sT * sT) + dm * dm / (sm * sm));
    sup = 1.0 - std::exp(-ex);
  }
  for (int k = 0; k < 9; k++) kq[k] = sup * c.kappa_over_T2[k] * (T * T);
  for (int i = 0; i < 3; i++) tq[4 * i] += 0.2 / T;
}

// Per-particle output of the diffusion MRF assembly.
struct DiffMRF {
  double F0q[3], R0q[9], M0q[9];   // F_0_q_b (b), R_0_q_bc (3b + c), M_0_q_bj (3b + j)
  double Fq[9], Rq[27], Mq[27];    // F_q_ib (3i + b), R_q_ibc (9i + 3b + c), M_q_ibj (9i + 3b + j)
};

// src/eom_default.cpp:1415-1817 (calculate_MRF_diffusion) for one particle
// (D = 2, 3; Milne coordinates). Ms, Fs: M and F of the extensive entropy.
// The stray semicolon of :1744 ends F_D_ib after its second term; the two
// lines after it have no effect and are not restated.
void diffusion_mrf(const System& s, int a, double t, const double* Ms, double Fs, DiffMRF& o) {
  const int D = s.cfg.dim;
  // the Cartesian twin (src/eom_cartesian.cpp:1327-1722): metric without
  // tau, no F_D terms, expansion rate gamma div v
  const bool cart = s.cfg.coord == 1;
  const double t2 = cart ? 1.0 : t * t;
  const double sig = s.sigma[a], g = s.gamma[a], sden = s.th[kS][a], T = s.th[kT][a];
  const double rho[3] = {s.th[kRhoB][a], s.th[kRhoS][a], s.th[kRhoQ][a]};
  const double mu[3] = {s.th[kMuB][a], s.th[kMuS][a], s.th[kMuQ][a]};
  double das[3], dar[3][3], RS[3], MS[3] = {0, 0, 0}, ga[3][3] = {{0}}, q[3][4], qc[3][4];
  for (int c = 0; c < 3; c++) {
    das[c] = s.dalpha[c][a];
    for (int d = 0; d < 3; d++) dar[c][d] = s.dalpha[3 + 3 * c + d][a];
    RS[c] = -mu[c] / T;
    for (int m = 0; m < 4; m++) q[c][m] = s.q[4 * c + m][a];
    qc[c][0] = q[c][0];
    qc[c][1] = -q[c][1];
    qc[c][2] = -q[c][2];
    qc[c][3] = -t2 * q[c][3];
  }
  double u[3] = {0, 0, 0}, uc[3], fu[3] = {0, 0, 0}, divV = 0;
  for (int i = 0; i < D; i++) {
    u[i] = s.u[i][a];
    fu[i] = u[i];
    MS[i] = Ms[i];
    divV += s.gradV[i * D + i][a];
    for (int c = 0; c < 3; c++) ga[i][c] = s.grad_alpha[3 * i + c][a];
  }
  for (int i = 0; i < 3; i++) uc[i] = u[i];
  cov_D(D, uc, t2);
  const double fuc[3] = {-fu[0], -fu[1], -t2 * fu[2]};
  const double geo = cart ? 0.0 : dEta(D, D - 1) * u[D - 1] * u[D - 1] * t / g;
  const double cmd[4] = {1., -1., -1., cart ? -1. : -1. / t / t};
  double tq[9], kq[9], itq[9], itt[9], itk[9];
  for (int k = 0; k < 9; k++) { tq[k] = s.tau_q[k][a]; kq[k] = s.kappa_q[k][a]; }
  inverse(3, tq, itq);
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++) {
      itt[3 * c + d] = 0.0;
      itk[3 * c + d] = 0.0;
      for (int k = 0; k < 3; k++) {
        itt[3 * c + d] += itq[3 * c + k] * tq[3 * k + d];
        itk[3 * c + d] += itq[3 * c + k] * kq[3 * k + d];
      }
    }
  const double X = cart ? g * divV : g * divV + geo + g / t;
  const double omg = 1. - g * g;
  // the 0 (time) components
  double F0D[3], F0a[3], A0a[3], R0a[3][3], M0a[3][3] = {{0}}, M0D[3][3] = {{0}};
  for (int c = 0; c < 3; c++) {
    F0D[c] = cart ? 0.0
                  : g * g * geo * q[c][0] + 2. * g * g * qc[c][3] * fu[2] / t + t * g * qc[c][0] * fu[2] * fu[2] +
                        t * fu[2] * q[c][3];
    F0a[c] = omg * sig * das[c] * Fs;
    A0a[c] = -omg * das[c] * sden / g;
    for (int i = 0; i < D; i++) {
      M0D[c][i] = g * g * (qc[c][i + 1] - qc[c][0] * uc[i] / g);
      M0a[c][i] = omg * sig * das[c] * MS[i];
      F0a[c] += -ga[i][c] * u[i] / g;
    }
    for (int d = 0; d < 3; d++) {
      R0a[c][d] = omg * sig * (das[c] * RS[d] + dar[c][d]);
      A0a[c] += -omg * dar[c][d] * rho[d] / g;
    }
  }
  for (int c = 0; c < 3; c++) {
    o.F0q[c] = 0.0;
    for (int i = 0; i < 3; i++) o.M0q[3 * c + i] = 0.0;
    for (int i = 0; i < D; i++) {
      double acc = 0;
      for (int d = 0; d < 3; d++)
        acc += (-itt[3 * c + d] * M0D[d][i] + itk[3 * c + d] * M0a[d][i] - itk[3 * c + d] * A0a[d] * uc[i] / g) / (g) +
               itt[3 * c + d] * q[d][0] * uc[i] / g / g;
      o.M0q[3 * c + i] = acc;
    }
    for (int d = 0; d < 3; d++)
      o.F0q[c] += (-itt[3 * c + d] * F0D[d] - itq[3 * c + d] * q[d][0] + itk[3 * c + d] * F0a[d] +
                   itk[3 * c + d] * A0a[d] * X) / (g) -
                  itt[3 * c + d] * q[d][0] * X / g;
    for (int d = 0; d < 3; d++) {
      double acc = 0.0;
      for (int k = 0; k < 3; k++) acc += itk[3 * c + k] * R0a[k][d] / (g);
      o.R0q[3 * c + d] = acc;
    }
  }
  // the spatial components, all three directions
  double FD[3][3], Fa[3][3], Aa[3][3], MD[3][3][3], Ma[3][3][3], Ra[3][3][3];
  for (int i = 0; i < 3; i++)
    for (int c = 0; c < 3; c++) {
      FD[i][c] = cart ? 0.0 : fu[i] * g * q[c][0] * geo + 2. * fu[i] * qc[c][3] * fu[2] * g / t;
      Fa[i][c] = -fu[i] * g * sig * das[c] * Fs + cmd[i + 1] * ga[i][c];
      Aa[i][c] = fu[i] * das[c] * sden;
      for (int j = 0; j < 3; j++) {
        MD[i][c][j] = fu[i] * g * (qc[c][j + 1] - qc[c][0] * fuc[j] / g);
        Ma[i][c][j] = -fu[i] * g * sig * das[c] * MS[j];
      }
      for (int d = 0; d < 3; d++) {
        Ra[i][c][d] = -fu[i] * g * sig * (das[c] * RS[d] + dar[c][d]);
        Aa[i][c] += fu[i] * dar[c][d] * rho[d];
      }
    }
  for (int i = 0; i < 3; i++)
    for (int c = 0; c < 3; c++) {
      double F = 0.0;
      for (int d = 0; d < 3; d++) {
        F += (-itt[3 * c + d] * FD[i][d] - itq[3 * c + d] * q[d][i + 1] + itk[3 * c + d] * Fa[i][d] +
              itk[3 * c + d] * Aa[i][d] * X) / (g * sig);
        double R = 0.0;
        for (int k = 0; k < 3; k++) R += itk[3 * c + k] * Ra[i][k][d] / (g * sig);
        o.Rq[9 * i + 3 * c + d] = R;
      }
      o.Fq[3 * i + c] = F;
      for (int j = 0; j < 3; j++) {
        double M = 0.0;
        for (int d = 0; d < 3; d++)
          M += (-itt[3 * c + d] * MD[i][d][j] + itk[3 * c + d] * Ma[i][d][j] - itk[3 * c + d] * Aa[i][d] * fuc[j] / g) /
               (g * sig);
        o.Mq[9 * i + 3 * c + j] = M;
      }
    }
}

// Per-particle output of the shear MRF assembly.
struct ShearMRF {
  double M0i[9], F0i[3], Mnab[3], Fnab;
  double Mext[2][3][3], Fext[2][3];
  double Msig[2][3][3], Fsig[2][3];   // M_sigma, F_sigma of the shear tensor sigma^{ij}
};

// src/eom_default.cpp:882-1412 (calculate_MRF_shear) for one particle.
void shear_mrf(const System& s, int a, double t, bool use_vort, ShearMRF& o) {
  const int D = s.cfg.dim;
  // Cartesian (src/eom_cartesian.cpp:840-1400): the metric without tau and
  // none of the Milne connection terms (1/tau, the geometric factor, eta deltas)
  const bool cart = s.cfg.coord == 1;
  const double tm = cart ? 1.0 : t, ch = cart ? 0.0 : 1.0;
  auto dE = [&](int i) { return cart ? 0.0 : dEta(D, i); };
  const double t2 = tm * tm;
  const double cmd[4] = {1.0, -1.0, -1.0, -1.0 / tm / tm};
  const double sigma = s.sigma[a], g = s.gamma[a];
  const double eta = s.eta_pi[a], phi6 = s.phi6[a], phi7 = s.phi7[a], lpP = s.lambda_piPi[a];
  const double tpp = s.tau_pipi[a], dpp = s.delta_pipi[a], tpi = s.tau_pi[a];
  const double tdelta = dpp - tpi;
  const double Pi = s.bulk[a];
  double u[3] = {0, 0, 0}, uc[3], v[3] = {0, 0, 0}, fu[3] = {0, 0, 0}, fuc[3];
  for (int i = 0; i < D; i++) { u[i] = s.u[i][a]; v[i] = s.v[i][a]; fu[i] = u[i]; }
  for (int i = 0; i < 3; i++) { uc[i] = u[i]; fuc[i] = fu[i]; }
  cov_D(D, uc, t2);
  fuc[0] = -fuc[0]; fuc[1] = -fuc[1]; fuc[2] *= -t2;  // Vector<3> make_covariant
  double pi[4][4], hy[4][4], pc[4][4];
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) pi[i][j] = s.shv[i * 4 + j][a];
  // shv_hybrid = pi^mu_nu (Matrix<4,4>::make_covariant slot 1), shv_cov slot 0 on top
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) {
      double f = (j == 1 || j == 2) ? -1.0 : (j == 3 ? -t2 : 1.0);
      hy[i][j] = pi[i][j] * f;
    }
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) {
      double f = (i == 1 || i == 2) ? -1.0 : (i == 3 ? -t2 : 1.0);
      pc[i][j] = hy[i][j] * f;
    }
  const double geo = dE(D - 1) * u[D - 1] * u[D - 1] * t / g;
  const double gt = cart ? 0.0 : g / t;
  double gV[3][3] = {{0}}, divV = 0;
  for (int i = 0; i < D; i++) {
    divV += s.gradV[i * D + i][a];
    for (int j = 0; j < D; j++) gV[i][j] = s.gradV[i * D + j][a];
  }
  double gu[3][3] = {{0}}, gu0[3] = {0, 0, 0};
  for (int i = 0; i < D; i++)
    for (int j = 0; j < D; j++) {
      gu[i][j] = g * gV[i][j];
      for (int k = 0; k < D; k++) gu[i][j] += -g * u[j] * uc[k] * gV[i][k];
    }
  for (int i = 0; i < D; i++) {
    double acc = 0;
    for (int j = 0; j < D; j++) acc += gu[i][j] * uc[j];
    gu0[i] = -1. * acc / g;
  }
  double gu0c[3] = {gu0[0], gu0[1], gu0[2]};
  contra_D(D, gu0c, t2);
  double cgu[3][3] = {{0}};  // contravariant first index, zero padded to 3x3
  for (int i = 0; i < D; i++)
    for (int j = 0; j < D; j++) {
      double f = (D == 2) ? -1.0 : (i < D - 1 ? -1.0 : -1.0 / t2);
      cgu[i][j] = gu[i][j] * f;
    }
  double gu3[3][3] = {{0}};
  for (int i = 0; i < D; i++) for (int j = 0; j < D; j++) gu3[i][j] = gu[i][j];

  double guv[3] = {0, 0, 0};  // contract(grad_uj, v, FirstIndex)
  for (int j = 0; j < D; j++) for (int k = 0; k < D; k++) guv[j] += gu[k][j] * v[k];
  double gu0v = 0;
  for (int k = 0; k < D; k++) gu0v += gu0[k] * v[k];

  double v_gradu_shv[3], gugs[3], sgu[3], vsgu[3];
  for (int i = 0; i < D; i++) {
    v_gradu_shv[i] = 0.0;
    for (int j = 0; j < D; j++) v_gradu_shv[i] += guv[j] * hy[i + 1][j + 1];
    v_gradu_shv[i] += gu0v * hy[i + 1][0];
    gugs[i] = 0.0;
    for (int j = 0; j < D; j++) gugs[i] += cgu[i][j] * hy[0][j + 1];
    gugs[i] += cmd[i + 1] * gu0[i] * hy[0][0];
    sgu[i] = 0.0;
    for (int j = 0; j < D; j++) sgu[i] += pi[j + 1][0] * gu[j][i] + pi[j + 1][i + 1] * gu0[j];
    vsgu[i] = 0.0;
    for (int j = 0; j < D; j++) vsgu[i] += v[j] * pi[0][0] * gu[j][i] + v[j] * pi[0][i + 1] * gu0[j];
  }
  double sgu_s = 0.0;
  for (int i = 0; i < D; i++) {
    for (int j = 0; j < D; j++) sgu_s += (hy[i + 1][j + 1] - v[i] * hy[0][j + 1]) * gu[i][j];
    sgu_s += (hy[i + 1][0] - v[i] * hy[0][0]) * gu0[i];
  }
  double ss = 0.0;
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) ss += pi[i][j] * pc[i][j];
  double sl0[3];
  for (int i = 0; i < D; i++) {
    sl0[i] = 0.0;
    for (int j = 0; j < 4; j++) sl0[i] += (pi[0][j] * hy[i + 1][j] + pi[i + 1][j] * hy[0][j]) / 2.;
  }
  const double uD = u[D - 1];
  const double expn = geo + gt + g * divV;
  double Fs[3], FD[3], Fds[3], Fdo[3], Fdd[3], Ms[3][3], MD[3][3], Mds[3][3], Mdo[3][3], Mdd[3][3];
  for (int i = 0; i < D; i++) {
    const double di = dE(i);
    Fs[i] = -(guv[i] - gu0c[i]) / 2. + u[i] * g * (geo + gt + g * divV) / 3. - g * geo * u[i] / 2.;
    FD[i] = g * (u[i] * hy[0][0] + g * hy[i + 1][0]) * geo + t * uD * pi[3][i + 1] * di;
    Fds[i] = -(v_gradu_shv[i] - gugs[i] - 4. * g * u[i] * sgu_s / 3. - sgu[i] + vsgu[i]) / 4. +
             (hy[i + 1][0] - g * g * hy[i + 1][0] - g * u[i] * hy[0][0] + pi[0][i + 1] +
              4. * u[i] * g * hy[0][0] / 3.) * geo / 4. +
             ch * (g * cmd[i + 1] * hy[0][3] * di / t + g * pi[3][0] * di / t +
                   4. * g * u[i] * (g * hy[3][3] / t) / 3.) / 4. -
             pi[0][i + 1] * (gt + geo + g * divV) / 3.;
    Fdo[i] = -(v_gradu_shv[i] - gugs[i] + sgu[i] - vsgu[i]) / 4. +
             (hy[i + 1][0] - g * g * hy[i + 1][0] - g * u[i] * hy[0][0] - pi[0][i + 1]) * geo / 4. +
             ch * (g * cmd[i + 1] * hy[0][3] * di / t - g * pi[3][0] * di / t) / 4.;
    Fdd[i] = pi[i + 1][0] * expn;
    for (int j = 0; j < D; j++) {
      Ms[i][j] = u[i] * uc[j] / (2. * 3.);
      MD[i][j] = g * u[i] * (hy[0][j + 1] - hy[0][0] * uc[j] / g) + g * g * (hy[i + 1][j + 1] - hy[i + 1][0] * uc[j] / g);
      Mds[i][j] = (hy[i + 1][j + 1] - hy[i + 1][0] * uc[j] / g - g * g * hy[i + 1][j + 1] - g * u[i] * hy[0][j + 1] +
                   uc[j] * g * hy[i + 1][0] + uc[j] * u[i] * hy[0][0] +
                   4. * g * u[i] * (hy[0][j + 1] - hy[0][0] * uc[j] / g) / 3. +
                   (-pi[0][i + 1] + 4. * pi[0][i + 1] / 3.) * uc[j] / g) / 4.;
      Mdo[i][j] = (hy[i + 1][j + 1] - hy[i + 1][0] * uc[j] / g - g * g * hy[i + 1][j + 1] - g * u[i] * hy[0][j + 1] +
                   uc[j] * g * hy[i + 1][0] + uc[j] * u[i] * hy[0][0] + pi[0][i + 1] * uc[j] / g) / 4.;
      Mdd[i][j] = -pi[i + 1][0] * uc[j] / g;
    }
    Ms[i][i] += (1. - g * g) / 2.;
    Mdo[i][i] += -pi[0][0] / 4.;
    Mds[i][i] += +pi[0][0] / 4.;
    Fs[i] += di * (-(-uD * t - uD / t + g * uD * uD * t + 2. * g * g * uD / t) / 2.);
    FD[i] += di * (uD * pi[0][0] / t + g * pi[3][0] / t);
    if (D != 2 && !cart) {
      Fds[i] += (t * uD * di * cmd[i + 1] * hy[0][0] + uD * hy[i + 1][3] * g / t / 4. + hy[i + 1][3] * t * uD +
                 pi[0][0] * di * uD / t + t * uD * uD * (g * hy[i + 1][0] + u[i] * hy[0][0]) +
                 2. * g * uD * (g * hy[i + 1][3] + u[i] * pi[0][3]) / t) / 4. +
                g * u[i] * (hy[3][0] * uD * t + uD * hy[0][3] / t) / 3.;
      Fdo[i] += (t * uD * di * cmd[i + 1] * hy[0][0] + uD * hy[i + 1][3] * g / t - hy[3][i + 1] * t * uD -
                 pi[0][0] * di * uD / t + t * uD * uD * (g * hy[i + 1][0] + u[i] * hy[0][0]) +
                 2. * g * uD * (g * hy[i + 1][3] + u[i] * pi[0][3]) / t) / 4.;
    }
  }
  double Fnab = 0.0;
  for (int i = 0; i < D; i++) {
    o.Mnab[i] = hy[0][i + 1] - hy[0][0] * uc[i] / g;
    for (int j = 0; j < D; j++) Fnab += (hy[i + 1][j + 1] - v[i] * hy[0][j + 1]) * gu[i][j];
    Fnab += (hy[i + 1][0] - v[i] * hy[0][0]) * gu0[i];
  }
  Fnab += +ch * (hy[3][3] * g / t) + hy[0][0] * geo + (t * hy[3][0] + hy[0][3] / t) * uD * dE(D - 1);
  o.Fnab = Fnab;
  const double uv = use_vort ? 1.0 : 0.0;
  for (int i = 0; i < D; i++) {
    o.F0i[i] = (-pi[i + 1][0] - tpi * FD[i] - dpp * Fdd[i] + 2. * tpi * Fdo[i] * uv - tpp * Fds[i] +
                (2. * eta + lpP * Pi) * Fs[i] + phi6 * Pi * pi[i + 1][0] + phi7 * (sl0[i] + g * u[i] * ss / 3.)) /
               (tpi * g);
    for (int j = 0; j < D; j++)
      o.M0i[i * D + j] = (-tpi * MD[i][j] - dpp * Mdd[i][j] + 2. * tpi * Mdo[i][j] * uv - tpp * Mds[i][j] +
                          (2. * eta + lpP * Pi) * Ms[i][j]) / (tpi * g);
  }
  // shear-tensor evolution (2x3 upper block, i <= j)
  double gugjs[2][3], sigu[2][3], vsig[2][3], sml[2][3];
  for (int i = 0; i < 2; i++)
    for (int j = i; j < 3; j++) {
      gugjs[i][j] = sigu[i][j] = vsig[i][j] = sml[i][j] = 0.0;
      for (int k = 0; k < D; k++) {
        gugjs[i][j] += cgu[i][k] * hy[j + 1][k + 1] + cgu[j][k] * hy[i + 1][k + 1];
        sigu[i][j] += pi[k + 1][i + 1] * gu3[k][j] + pi[k + 1][j + 1] * gu3[k][i];
        vsig[i][j] += v[k] * pi[0][i + 1] * gu3[k][j] + v[k] * pi[0][j + 1] * gu3[k][i];
      }
      for (int k = 0; k < 4; k++) sml[i][j] += (pi[i + 1][k] * hy[j + 1][k] + pi[j + 1][k] * hy[i + 1][k]) / 2.;
    }
  double FD2[2][3] = {{0}}, Fsg[2][3] = {{0}}, Fdl[2][3] = {{0}}, Fdo2[2][3] = {{0}}, Fds2[2][3] = {{0}};
  double MD2[2][3][3] = {{{0}}}, Msg[2][3][3] = {{{0}}}, Mdl[2][3][3] = {{{0}}}, Mdo2[2][3][3] = {{{0}}},
         Mds2[2][3][3] = {{{0}}};
  const double f2 = fu[2];
  for (int i = 0; i < 2; i++) {
    for (int j = i; j < 3; j++) {
      const double di = dE(i), dj = dE(j);
      FD2[i][j] = g * geo * (fu[i] * hy[j + 1][0] + fu[j] * hy[i + 1][0]);
      Fsg[i][j] = cgu[i][j] / 2. + cgu[j][i] / 2. + fu[i] * fu[j] * expn / 3.;
      Fdl[i][j] = pi[i + 1][j + 1] * expn;
      const double common = ch *
          (t * f2 * (cmd[i + 1] * hy[j + 1][0] * di + cmd[j + 1] * hy[i + 1][0] * dj) +
          g * (cmd[i + 1] * hy[j + 1][3] * di + cmd[j + 1] * hy[i + 1][3] * dj) / t +
          f2 * f2 * t * (fu[i] * hy[j + 1][0] + fu[j] * hy[i + 1][0]) +
          2. * g * f2 * (fu[i] * hy[j + 1][3] + fu[j] * hy[i + 1][3]) / t);
      const double cross = ch * (g * (pi[3][i + 1] * dj + pi[3][j + 1] * di) / t +
                                 f2 * (pi[0][i + 1] * dj + pi[0][j + 1] * di) / t);
      Fdo2[i][j] = -(-gugjs[i][j] + sigu[i][j] - vsig[i][j]) / 4. +
                   (-fu[i] * g * hy[j + 1][0] - fu[j] * g * hy[i + 1][0]) * geo / 4. + (common - cross) / 4.;
      Fds2[i][j] = -(-gugjs[i][j] - sigu[i][j] + vsig[i][j] - 4. * (fu[i] * fu[j]) * sgu_s / 3.) / 4. +
                   (-fu[i] * g * hy[j + 1][0] - fu[j] * g * hy[i + 1][0] + 4. * fu[i] * fu[j] * hy[0][0] / 3.) * geo / 4. +
                   (common + cross +
                    ch * (4. * fu[i] * fu[j] * (hy[3][0] * f2 * t + g * hy[3][3] / t + f2 * hy[0][3] / t) / 3.)) / 4. -
                   pi[i + 1][j + 1] * (gt + geo + g * divV) / 3.;
      for (int k = 0; k < D; k++) {
        MD2[i][j][k] = g * (fu[i] * hy[j + 1][k + 1] - fu[i] * hy[j + 1][0] * fuc[k] / g + fu[j] * hy[i + 1][k + 1] -
                            fu[j] * hy[i + 1][0] * fuc[k] / g);
        Msg[i][j][k] = -fu[i] * fu[j] * fuc[k] / (3. * g);
        Mdl[i][j][k] = -pi[i + 1][j + 1] * fuc[k] / g;
        Mdo2[i][j][k] = (-fu[i] * hy[j + 1][k + 1] * g - fu[j] * hy[i + 1][k + 1] * g + fuc[k] * fu[i] * hy[j + 1][0] +
                         fuc[k] * fu[j] * hy[i + 1][0]) / 4.;
        Mds2[i][j][k] = (-fu[i] * hy[j + 1][k + 1] * g - fu[j] * hy[i + 1][k + 1] * g + fuc[k] * fu[i] * hy[j + 1][0] +
                         fuc[k] * fu[j] * hy[i + 1][0] +
                         4. * fu[i] * fu[j] * (hy[0][k + 1] - hy[0][0] * fuc[k] / g) / 3. +
                         4. * pi[i + 1][j + 1] * fuc[k] / 3. / g) / 4.;
      }
      Mds2[i][j][i] += pi[0][j + 1] / 4.;
      Mdo2[i][j][i] += -pi[0][j + 1] / 4.;
      Msg[i][j][i] += -g * fu[j] / 2.;
    }
    for (int j = i; j < D; j++) {
      Msg[i][j][j] += -g * fu[i] / 2.;
      Mds2[i][j][j] += pi[0][i + 1] / 4.;
      Mdo2[i][j][j] += -pi[0][i + 1] / 4.;
    }
    for (int k = 0; k < D; k++) {
      Msg[i][i][k] += cmd[i + 1] * fuc[k] / (g * 3.);
      Mds2[i][i][k] += -cmd[i + 1] * (hy[0][k + 1] - hy[0][0] * fuc[k] / g) / 3.;
    }
    if (!cart) FD2[i][2] += g * pi[3][i + 1] / t + f2 * pi[0][i + 1] / t;
    Fsg[i][i] += -cmd[i + 1] * expn / 3.;
    if (!cart) Fsg[i][2] += -fu[i] * f2 * f2 * t / 2. - fu[i] * f2 * g / t;
    Fds2[i][i] += -cmd[i + 1] * sgu_s / 3. - cmd[i + 1] * hy[0][0] * geo / 3. -
                  ch * (cmd[i + 1] * (hy[3][0] * f2 * t + g * hy[3][3] / t + f2 * hy[0][3] / t) / 3.);
  }
  for (int i = 0; i < 2; i++) {
    for (int j = i; j < 3; j++) {
      o.Fext[i][j] = (-pi[i + 1][j + 1] - tdelta * Fdl[i][j] - tpi * FD2[i][j] + 2. * tpi * Fdo2[i][j] * uv -
                      tpp * Fds2[i][j] + (2. * eta + lpP * Pi) * Fsg[i][j] + phi6 * Pi * pi[i + 1][j + 1] +
                      phi7 * (sml[i][j] + fu[i] * fu[j] * ss / 3.)) / (sigma * tpi * g);
      for (int k = 0; k < D; k++)
        o.Mext[i][j][k] = (-tpi * MD2[i][j][k] - tdelta * Mdl[i][j][k] + 2. * tpi * Mdo2[i][j][k] * uv -
                           tpp * Mds2[i][j][k] + (2. * eta + lpP * Pi) * Msg[i][j][k]) / (sigma * tpi * g);
    }
    o.Fext[i][i] += phi7 * (-cmd[i + 1] * ss) / (3. * tpi * g * sigma);
  }
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 3; j++) {
      o.Fsig[i][j] = Fsg[i][j];
      for (int k = 0; k < 3; k++) o.Msig[i][j][k] = Msg[i][j][k];
    }
}

// src/eom_default.cpp:1831-1985 (compute_hydro_numbers), without the
// diffusion sector: the full sigma^{mu nu} from its five stored spatial
// entries (symmetry, orthogonality to u, tracelessness), the shear and bulk
// Knudsen numbers tau_pi sqrt|sigma:sigma| and tau_Pi |theta|, and the inverse
// Reynolds numbers sqrt|pi:pi| / p and |Pi| / p.
void hydro_numbers(System& s, int a, const double* sig5) {
  const int D = s.cfg.dim;
  const double t = s.cfg.coord == 1 ? 1.0 : s.t, t2 = t * t;
  const double g = s.gamma[a];
  double uc[3] = {0, 0, 0};
  for (int i = 0; i < D; i++) uc[i] = s.u[i][a];
  uc[0] = -uc[0];
  uc[1] = -uc[1];
  uc[2] *= -t2;
  double st[4][4] = {{0}};
  const int map[2][3] = {{0, 1, 2}, {-1, 3, 4}};
  for (int i = 0; i < 2; i++)
    for (int j = i; j < 3; j++) st[i + 1][j + 1] = sig5[map[i][j]];
  for (int i = 1; i < 4; i++)
    for (int j = i + 1; j < 4; j++) st[j][i] = st[i][j];
  for (int i = 1; i < D + 1; i++) {
    double c = 0.0;
    for (int j = 1; j < D + 1; j++) c += uc[j - 1] * st[i][j];
    st[0][i] = -1. * c / g;
  }
  for (int i = 1; i < 4; i++) st[i][0] = st[0][i];
  st[0][0] = (uc[0] * uc[0] * st[1][1] + uc[1] * uc[1] * st[2][2] + 2. * uc[1] * uc[0] * st[2][1] +
              2. * uc[2] * uc[0] * st[3][1] + 2. * uc[2] * uc[1] * st[3][2] -
              uc[2] * uc[2] * (st[1][1] + st[2][2]) / t2) /
             (g * g - uc[2] * uc[2] / t2);
  st[3][3] = (st[0][0] - st[1][1] - st[2][2]) / t2;
  const double gm[4] = {1.0, -1.0, -1.0, -t2};
  double sn = 0.0, pn = 0.0;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      sn += st[i][j] * (st[i][j] * gm[j] * gm[i]);
      pn += s.shv[i * 4 + j][a] * (s.shv[i * 4 + j][a] * gm[j] * gm[i]);
    }
  const double p = s.th[kP][a];
  for (int k = 0; k < 5; k++) s.sigma_t[k][a] = sig5[k];
  s.kn_shear[a] = s.tau_pi[a] * std::sqrt(std::fabs(sn));
  s.kn_bulk[a] = s.tau_Pi[a] * std::fabs(s.theta[a]);
  s.ire_shear[a] = std::sqrt(std::fabs(pn)) / p;
  s.ire_bulk[a] = std::fabs(s.bulk[a]) / p;
}

// src/eom_default.cpp:1944-1982: per charge, Kn = tau_q^{aa} |grad alpha_a|
// and the inverse Reynolds number |q_a| / |n_a| (zero for |n_a| <= 1e-15).
void diffusion_numbers(System& s, int a) {
  const int D = s.cfg.dim;
  const double t2 = s.cfg.coord == 1 ? 1.0 : s.t * s.t;
  const double rho[3] = {s.th[kRhoB][a], s.th[kRhoS][a], s.th[kRhoQ][a]};
  for (int c = 0; c < 3; c++) {
    double gsq = 0.0;
    for (int i = 0; i < D; i++) {
      const double gg = s.grad_alpha[3 * i + c][a];
      gsq += gg * gg;
    }
    s.kn_diff[c][a] = s.tau_q[4 * c][a] * std::sqrt(gsq);
    const double q0 = s.q[4 * c][a], q1 = s.q[4 * c + 1][a], q2 = s.q[4 * c + 2][a], q3 = s.q[4 * c + 3][a];
    const double q_sq = q1 * q1 + q2 * q2 + t2 * q3 * q3 - q0 * q0;
    const double q_mag = q_sq > 0.0 ? std::sqrt(q_sq) : 0.0;
    const double n_abs = std::fabs(rho[c]);
    s.ire_diff[c][a] = (n_abs > 1e-15) ? q_mag / n_abs : 0.0;
  }
}

}  // namespace

// src/eom_default.cpp:17-38 (update_velocity)
void update_velocity(System& s) {
  const int D = s.cfg.dim;
  const double tm = s.cfg.coord == 1 ? 1.0 : s.t, t2 = tm * tm;
#pragma omp parallel for
  for (int a = 0; a < s.n; a++) {
    double u[3] = {s.u[0][a], s.u[1][a], s.u[2][a]};
    double g = gamma_of(D, u, t2);
    s.gamma[a] = g;
    for (int i = 0; i < D; i++) s.v[i][a] = u[i] / g;
  }
}

// src/eom_default.cpp:56-172 (reset_pi_tensor).
void reset_pi_tensor(System& s) {
  const int D = s.cfg.dim;
  const double tm = s.cfg.coord == 1 ? 1.0 : s.t, t2 = tm * tm;
#pragma omp parallel for
  for (int a = 0; a < s.n; a++) {
    const double g = s.gamma[a], sig = s.sigma[a];
    double fu[3] = {0, 0, 0};
    for (int i = 0; i < D; i++) fu[i] = s.u[i][a];
    double fc[3] = {-fu[0], -fu[1], -t2 * fu[2]};
    s.bulk[a] = s.ext_bulk[a] * sig;
    double p[4][4] = {{0}};
    const int map[2][3] = {{0, 1, 2}, {-1, 3, 4}};
    for (int i = 0; i < 2; i++)
      for (int j = i; j < 3; j++) p[i + 1][j + 1] = s.ext_shv[map[i][j]][a] * sig;
    for (int i = 1; i < 4; i++) for (int j = i + 1; j < 4; j++) p[j][i] = p[i][j];
    p[0][0] = (fc[0] * fc[0] * p[1][1] + fc[1] * fc[1] * p[2][2] + 2. * fc[1] * fc[0] * p[2][1] +
               2. * fc[2] * fc[0] * p[3][1] + 2. * fc[2] * fc[1] * p[3][2] - fc[2] * fc[2] * (p[1][1] + p[2][2]) / t2) /
              (g * g - fc[2] * fc[2] / (t2));
    p[3][3] = (p[0][0] - p[1][1] - p[2][2]) / t2;
    for (int i = 0; i < 3; i++) {
      double acc = 0.;
      for (int j = 0; j < 3; j++) acc += -p[i + 1][j + 1] * fc[j] / g;
      p[0][i + 1] = acc;
    }
    for (int i = 1; i < 4; i++) p[i][0] = p[0][i];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) s.shv[i * 4 + j][a] = p[i][j];
    // diffusion (:140-165): q^i = ext_q sigma, q^0 = -q^i u_i / gamma
    for (int c = 0; c < 3; c++) {
      double q0 = 0.;
      for (int i = 0; i < 3; i++) {
        const double qi = s.ext_q[3 * c + i][a] * sig;
        s.q[4 * c + i + 1][a] = qi;
      }
      for (int i = 0; i < 3; i++) q0 += -s.q[4 * c + i + 1][a] * fc[i] / g;
      s.q[4 * c][a] = q0;
    }
  }
}

// src/sph_workstation.cpp:132-218 (regulate_diffusion, PhysRevC.98.034916
// Eqs. C6-C8): |q_a| is capped at rq_max |n_a| f(e), f(e) = chi0 (Fermi(e) -
// Fermi(0)), Fermi(e) = 1 / (exp(-(e - e0) / xi0) + 1); the capped q^mu
// rescales all four components and the extensive current follows.
void regulate_diffusion(System& s) {
  if (!s.cfg.using_diffusion || !s.cfg.diffusion_regulator) return;
  const double chi0 = s.cfg.reg_chi0, e0 = s.cfg.reg_e0 / kHbarcGeVfm, xi0 = s.cfg.reg_xi0 / kHbarcGeVfm;
  const double rq_max = s.cfg.reg_rq_max;
  const double fermi_offset = 1.0 / (std::exp(e0 / xi0) + 1.0);
  const bool milne = s.cfg.coord == 0;
  const double t2 = s.t * s.t;
#pragma omp parallel for
  for (int a = 0; a < s.n; a++) {
    const double e = s.th[kE][a];
    const double ferm = 1.0 / (std::exp(-(e - e0) / xi0) + 1.0);
    const double f_str = chi0 * (ferm - fermi_offset);
    const double sigma = s.sigma[a];
    const double rho[3] = {s.th[kRhoB][a], s.th[kRhoS][a], s.th[kRhoQ][a]};
    for (int c = 0; c < 3; c++) {
      const double n_abs = std::fabs(rho[c]);
      if (n_abs < 1.0e-15) continue;
      const double q0 = s.q[4 * c][a], q1 = s.q[4 * c + 1][a], q2 = s.q[4 * c + 2][a], q3 = s.q[4 * c + 3][a];
      const double q3_sq = milne ? t2 * q3 * q3 : q3 * q3;
      const double q_sq = q1 * q1 + q2 * q2 + q3_sq - q0 * q0;
      if (q_sq <= 0.0) continue;
      const double q_mag = std::sqrt(q_sq);
      const double threshold = rq_max * n_abs * f_str;
      if (q_mag <= threshold) continue;
      const double scale = threshold / q_mag;
      s.q[4 * c][a] = q0 * scale;
      s.q[4 * c + 1][a] = q1 * scale;
      s.q[4 * c + 2][a] = q2 * scale;
      s.q[4 * c + 3][a] = q3 * scale;
      for (int i = 0; i < 3; i++) s.ext_q[3 * c + i][a] = s.q[4 * c + i + 1][a] / sigma;
    }
  }
}

// src/sph_workstation.cpp:1622-1699 (update_all_particle_viscosities)
void update_viscosities(System& s) {
#pragma omp parallel for
  for (int a = 0; a < s.n; a++) {
    double th[16];
    for (int k = 0; k < 16; k++) th[k] = s.th[k][a];
    Coefs k = coefs(s.cfg, th);
    s.eta_pi[a] = k.eta; s.tau_pi[a] = k.tau_pi; s.zeta_Pi[a] = k.zeta; s.tau_Pi[a] = k.tau_Pi;
    s.delta_PiPi[a] = k.delta_PiPi; s.delta_pipi[a] = k.delta_pipi; s.lambda_piPi[a] = k.lambda_piPi;
    s.lambda_Pipi[a] = k.lambda_Pipi; s.phi1[a] = k.phi1; s.phi3[a] = k.phi3; s.phi6[a] = k.phi6;
    s.phi7[a] = k.phi7; s.tau_pipi[a] = k.tau_pipi;
    if (s.cfg.using_diffusion) {
      double tq[9], kq[9];
      diffusion_coefs(s.cfg, th, s.cfg.eos_kind == kTable && s.eos_id[a] == 0, tq, kq);
      for (int j = 0; j < 9; j++) { s.tau_q[j][a] = tq[j]; s.kappa_q[j][a] = kq[j]; }
    }
  }
}

// src/sph_workstation.cpp:1713-1772 -> :658-741 (locate_phase_diagram_point_sBSQ):
// previous (T, mu) and EoS as the seed; thermo set from the solution.
int update_thermodynamics(System& s) {
  int failures = 0;
#pragma omp parallel for reduction(+ : failures)
  for (int a = 0; a < s.n; a++) {
    double x[4] = {s.th[kT][a], s.th[kMuB][a], s.th[kMuQ][a], s.th[kMuS][a]};
    double tgt[4] = {s.th[kS][a], s.th[kRhoB][a], s.th[kRhoS][a], s.th[kRhoQ][a]};
    int it = 0;
    int k = eos_invert(s.cfg, s.table, 1, tgt, s.eos_id[a], x, &it);
    if (k < 0) { s.eos_status[a] = -1; failures++; continue; }
    double th[16];
    eos_set_thermo(s.cfg, s.table, k, x, th);
    for (int j = 0; j < 16; j++) s.th[j][a] = th[j];
    s.eos_id[a] = k;
    s.eos_status[a] = it;
    if (s.cfg.using_diffusion) {
      double da[12];
      eos_alpha_derivs(s.cfg, s.table, k, x, da);
      for (int j = 0; j < 12; j++) s.dalpha[j][a] = da[j];
    }
  }
  return failures;
}

// src/eom_default.cpp:211-869 (evaluate_time_derivatives) without sources,
// with the diffusion sector when it is on (dN/dt is zero otherwise); with
// coord = 1 its Cartesian twin src/eom_cartesian.cpp:210-840 (no tau in the
// metric, no connection terms).
void evaluate_time_derivatives(System& s) {
  const int D = s.cfg.dim;
  const bool cart = s.cfg.coord == 1;
  const double t = s.t, tm = cart ? 1.0 : t, t2 = tm * tm;
  auto dE = [&](int i) { return cart ? 0.0 : dEta(D, i); };
  const bool shear = s.cfg.using_shear;
#pragma omp parallel for
  for (int a = 0; a < s.n; a++) {
    ShearMRF sm{};
    if (shear) shear_mrf(s, a, t, s.cfg.using_vorticity, sm);
    const double g = s.gamma[a], sig = s.sigma[a];
    const double dwds = s.th[kDwds][a], T = s.th[kT][a], w = s.th[kW][a], sden = s.th[kS][a];
    const double rho[3] = {s.th[kRhoB][a], s.th[kRhoS][a], s.th[kRhoQ][a]};
    const double dwdr[3] = {s.th[kDwdB][a], s.th[kDwdS][a], s.th[kDwdQ][a]};
    const double mu[3] = {s.th[kMuB][a], s.th[kMuS][a], s.th[kMuQ][a]};
    const double Pi = s.bulk[a], zeta = s.zeta_Pi[a], tPi = s.tau_Pi[a], dPP = s.delta_PiPi[a];
    const double phi1 = s.phi1[a], phi3 = s.phi3[a], lPp = s.lambda_Pipi[a];
    const double ztil = zeta + (dPP - tPi) * Pi;
    double u[3] = {0, 0, 0}, uc[3];
    for (int i = 0; i < D; i++) u[i] = s.u[i][a];
    for (int i = 0; i < 3; i++) uc[i] = u[i];
    cov_D(D, uc, t2);
    double pi[4][4], pc[4][4];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) pi[i][j] = s.shv[i * 4 + j][a];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) {
        double fj = (j == 1 || j == 2) ? -1.0 : (j == 3 ? -t2 : 1.0);
        double fi = (i == 1 || i == 2) ? -1.0 : (i == 3 ? -t2 : 1.0);
        pc[i][j] = pi[i][j] * fj * fi;
      }
    double divV = 0;
    for (int i = 0; i < D; i++) divV += s.gradV[i * D + i][a];
    const double geo = dE(D - 1) * u[D - 1] * u[D - 1] * t / g;
    const double gt = cart ? 0.0 : g / t;
    const double expn = g * divV + gt + geo;
    // fill_auxiliary_variables (:229-362)
    double Mb[3], Ms[3];
    for (int i = 0; i < D; i++) {
      Mb[i] = (ztil * uc[i] / g) / (sig * g * tPi);
      Ms[i] = (Pi * uc[i] / g) / (sig * g * T);
    }
    // R_extensive_entropy = -mu/T multiplies dN/dt (zero without the
    // diffusion sector and sources)
    double RS[3];
    for (int c = 0; c < 3; c++) RS[c] = -mu[c] / T;
    double Fb = -(ztil * (g * divV + gt + geo) + Pi - phi1 * Pi * Pi) / (sig * g * tPi);
    double Fs = (-Pi * (g * divV + gt + geo)) / (sig * g * T);
    double Fnab = 0, Mnab[3] = {0, 0, 0};
    if (shear) {
      Fnab = sm.Fnab;
      Fs += Fnab / (sig * g * T);
      double pp = 0;
      for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) pp += pc[i][j] * pi[i][j];
      Fb += -(lPp * Fnab - phi3 * pp) / (sig * g * tPi);
      for (int i = 0; i < D; i++) {
        Mnab[i] = sm.Mnab[i];
        Mb[i] += -lPp * Mnab[i] / (sig * g * tPi);
        Ms[i] += Mnab[i] / (sig * g * T);
      }
    }
    // compute_velocity_derivative (:456-618)
    double gP[3], gB[3];
    for (int i = 0; i < D; i++) { gP[i] = s.gradP[i][a]; gB[i] = s.gradBulk[i][a]; }
    contra_D(D, gP, t2);
    contra_D(D, gB, t2);
    const double X = sden * dwds / g + (rho[0] * dwdr[0] + rho[1] * dwdr[1] + rho[2] * dwdr[2]) / g;
    double Mw[3];
    for (int i = 0; i < D; i++) Mw[i] = X * uc[i] / g + sig * dwds * Ms[i];
    const double Fw = -X * (geo + gt + g * divV) + sig * dwds * Fs;
    const double Fbulk = sig * Fb - Pi * (g * divV + gt + geo) / g;
    double Mu[9], Fu[3];
    for (int i = 0; i < D; i++) {
      for (int j = 0; j < D; j++) Mu[i * D + j] = u[i] * g * (Mb[j] + Mw[j]) - u[i] * uc[j] * (w + Pi) / g;
      Mu[i * D + i] += g * (w + Pi);
      Fu[i] = (gP[i] + gB[i]) - g * (Fw + Fbulk) * u[i] - (w + Pi) * expn * u[i];
      if (!cart) Fu[i] -= 2. * (w + Pi) * g * u[D - 1] * dEta(D, i) / t;
    }
    if (shear) {
      for (int i = 0; i < D; i++) {
        if (cart) Fu[i] += -s.divshear[i][a] + s.gradshear[i][a] - sm.F0i[i];
        else Fu[i] += -pi[i + 1][0] / t - 2. * dEta(D, i) * pi[0][3] / t - s.divshear[i][a] + s.gradshear[i][a] - sm.F0i[i];
        for (int j = 0; j < D; j++) Mu[i * D + j] += sm.M0i[i * D + j];
      }
    }
    // diffusion sector: the charge MRFs (compute_charge_derivative,
    // :368-451) and their coupling into du/dt (:579-617)
    const bool diff = s.cfg.using_diffusion;
    DiffMRF dm{};
    double RI[9], MN[3][3] = {{0}}, FN[3] = {0, 0, 0};
    if (diff) {
      diffusion_mrf(s, a, t, Ms, Fs, dm);
      double RN[9];
      for (int c = 0; c < 9; c++) RN[c] = 0.0;
      for (int c = 0; c < 3; c++) {
        RN[4 * c] += g * sig;
        FN[c] = 0.0;   // external charge sources
      }
      for (int i = 0; i < D; i++)
        for (int c = 0; c < 3; c++) MN[i][c] += -dm.M0q[3 * c + i];
      for (int c = 0; c < 3; c++) {
        for (int d = 0; d < 3; d++) RN[3 * c + d] += -dm.R0q[3 * c + d];
        if (cart) FN[c] += -dm.F0q[c] + s.grad_qa[c][a] - s.div_qa[c][a];
        else FN[c] += -dm.F0q[c] + s.grad_qa[c][a] - s.div_qa[c][a] - s.q[4 * c][a] / t;
      }
      inverse(3, RN, RI);
      // R_u = -u gamma (R_w + R_bulk sigma), R_w = sigma dw/drho + sigma dw/ds R_S;
      // R_bulk and the shear R_0i are zero
      double Ru[3][3];
      for (int i = 0; i < D; i++)
        for (int c = 0; c < 3; c++) {
          const double Rw = sig * dwdr[c] + sig * dwds * RS[c];
          Ru[i][c] = -u[i] * g * (Rw + 0.0 * sig);
        }
      double MR[9], FR[3];
      for (int i = 0; i < D; i++) {
        FR[i] = 0.0;
        for (int j = 0; j < D; j++) {
          MR[i * D + j] = 0.0;
          for (int c = 0; c < 3; c++)
            for (int d = 0; d < 3; d++) MR[i * D + j] += Ru[i][c] * RI[3 * c + d] * MN[j][d];
        }
        for (int c = 0; c < 3; c++)
          for (int d = 0; d < 3; d++) FR[i] += Ru[i][c] * RI[3 * c + d] * FN[d];
      }
      for (int i = 0; i < D; i++) {
        for (int j = 0; j < D; j++) Mu[i * D + j] = Mu[i * D + j] - MR[i * D + j];
        Fu[i] = Fu[i] + FR[i];
      }
    }
    double MI[9], du[3];
    inverse(D, Mu, MI);
    for (int i = 0; i < D; i++) {
      du[i] = 0;
      for (int j = 0; j < D; j++) du[i] += MI[i * D + j] * Fu[j];
    }
    double dN[3] = {0, 0, 0};
    if (diff) {
      double MU[3];
      for (int c = 0; c < 3; c++) {
        MU[c] = 0.;
        for (int i = 0; i < D; i++) MU[c] += MN[i][c] * du[i];
      }
      for (int c = 0; c < 3; c++) {
        dN[c] = 0.;
        for (int d = 0; d < 3; d++) dN[c] += RI[3 * c + d] * (FN[d] + MU[d]);
      }
      for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) {
          double v = dm.Fq[3 * i + c];
          for (int j = 0; j < D; j++) v += dm.Mq[9 * i + 3 * c + j] * du[j];
          for (int d = 0; d < 3; d++) v += dm.Rq[9 * i + 3 * c + d] * dN[d];
          s.d_ext_q[3 * c + i][a] = v;
        }
    }
    // compute_derivatives (:622-826)
    // contractions with du/dt first, then the F terms, as in the reference
    double m1 = 0, m2 = 0, m3 = 0, c1 = 0;
    for (int i = 0; i < D; i++) { m1 += Ms[i] * du[i]; m2 += Mb[i] * du[i]; m3 += Mnab[i] * du[i]; c1 += uc[i] * du[i]; }
    double rdn = 0.0;
    for (int c = 0; c < 3; c++) rdn += RS[c] * dN[c];
    const double dS = diff ? m1 + Fs + rdn : m1 + Fs, dB = m2 + Fb, snu = m3 + Fnab;
    const double th = -1. * c1 / g + g * divV + gt + geo;
    for (int i = 0; i < D; i++) s.du_dt[i][a] = du[i];
    s.d_ext[0][a] = dS;
    for (int c = 0; c < 3; c++) s.d_ext[1 + c][a] = dN[c];
    s.d_ext_bulk[a] = dB;
    s.theta[a] = th;
    s.shv_nabla_u[a] = snu;
    if (shear) {
      const int map[2][3] = {{0, 1, 2}, {-1, 3, 4}};
      double sig5[5];
      for (int i = 0; i < 2; i++)
        for (int j = i; j < 3; j++) {
          double acc = 0.;
          for (int k = 0; k < D; k++) acc += sm.Mext[i][j][k] * du[k];
          s.d_ext_shv[map[i][j]][a] = acc + sm.Fext[i][j];
          double as = 0.;
          for (int k = 0; k < D; k++) as += sm.Msig[i][j][k] * du[k];
          sig5[map[i][j]] = as + sm.Fsig[i][j];
        }
      hydro_numbers(s, a, sig5);
    } else {
      for (int k = 0; k < 6; k++) s.d_ext_shv[k][a] = 0.0;
      if (diff) {
        // the numbers are computed with shear or diffusion (:865-867); without
        // shear the stored sigma tensor stays zero
        const double zero5[5] = {0, 0, 0, 0, 0};
        hydro_numbers(s, a, zero5);
      }
    }
    if (diff) diffusion_numbers(s, a);
    // compute_Ez_derivative (:827-862)
    const double u3 = (D == 3) ? u[2] : 0.0;
    const double e = s.th[kE][a], p = s.th[kP][a];
    s.dEz[a] = ((e + p + Pi) * u3 * u3 + (p + Pi) / t2 + pi[3][3]) * s.mass[0][a] * t2 / s.sigma_lab[a];
  }
}

// src/sph_workstation.cpp:1509-1612 (get_time_derivatives), phases 01-10.
void get_time_derivatives(System& s, NbrList& nl) {
  build_neighbours(s, nl);        // 01_neighbour_list
  update_velocity(s);             // 02_gamma_velocity
  smooth_fields(s, nl);           // 03_smooth_fields
  update_thermodynamics(s);       // 04_thermodynamics
  reset_pi_tensor(s);             // 05_reset_pi_tensor
  regulate_diffusion(s);          // 06_regulate_diffusion
  update_viscosities(s);          // 08_viscosities
  smooth_gradients(s, nl);        // 09_smooth_gradients
  evaluate_time_derivatives(s);   // 10_time_derivatives
}

// src/evolver.cpp:124-168 (fill_cache), :344-486 (step_rk), :493-517 (rk2).
static void step_rk(System& s, NbrList& nl, double dt, double t0) {
  get_time_derivatives(s, nl);
  const int D = s.cfg.dim;
#pragma omp parallel for
  for (int a = 0; a < s.n; a++) {
    double es = s.ext0[0][a] + dt * s.d_ext[0][a];
    s.ext_bulk[a] = s.ext_bulk0[a] + dt * s.d_ext_bulk[a];
    for (int k = 1; k < 4; k++) s.ext[k][a] = s.ext0[k][a] + dt * s.d_ext[k][a];
    s.Ez[a] = s.Ez0[a] + dt * s.dEz[a];
    for (int i = 0; i < D; i++) {
      s.r[i][a] = s.r0[i][a] + dt * s.v[i][a];
      s.u[i][a] = s.u0[i][a] + dt * s.du_dt[i][a];
    }
    for (int k = 0; k < 5; k++) s.ext_shv[k][a] = s.ext_shv0[k][a] + dt * s.d_ext_shv[k][a];
    if (s.cfg.using_diffusion)
      for (int k = 0; k < 9; k++) s.ext_q[k][a] = s.ext_q0[k][a] + dt * s.d_ext_q[k][a];
    if (es < 0.0 && s.freeze[a] > 3) es = 1.e-3;
    else if (es < 0.0) s.eos_status[a] = -2;  // negative entropy: fatal in the reference
    s.ext[0][a] = es;
    for (int i = D; i < 3; i++) { s.r[i][a] = 0.0; s.u[i][a] = 0.0; }
  }
  s.t = t0 + dt;
}

void rk2_step(System& s, NbrList& nl) {
  for (int a = 0; a < s.n; a++) {
    for (int i = 0; i < 3; i++) { s.r0[i][a] = s.r[i][a]; s.u0[i][a] = s.u[i][a]; }
    for (int k = 0; k < 4; k++) s.ext0[k][a] = s.ext[k][a];
    s.ext_bulk0[a] = s.ext_bulk[a];
    for (int k = 0; k < 6; k++) s.ext_shv0[k][a] = s.ext_shv[k][a];
    for (int k = 0; k < 9; k++) s.ext_q0[k][a] = s.ext_q[k][a];
    s.Ez0[a] = s.Ez[a];
  }
  const double t0 = s.t, dt = s.cfg.dt;
  step_rk(s, nl, .5 * dt, t0);
  step_rk(s, nl, dt, t0);
  if (s.cfg.particlization) freeze_out_status(s);
}

// Freeze-out after a step (include/freeze_out.h; src/sph_workstation.cpp:1475-1486,
// freeze_out_particles): FreezeOut::check_freeze_out_status (:455-500), then
// bsqsvfreezeout (:549-615). Without cfg.surface only the energy of the
// snapshots is kept (what the status machine reads); with it every snapshot
// field, the backups of few-neighbour particles (freeze_out_evo, :322-375),
// and the hypersurface element of each particle that freezes
// (bsqsvinterpolate, :617-936), written as a freeze_out.dat row
// (src/output.cpp:417-482).
namespace {

void take_snapshot(const System& s, int a, double* out, int n) {
  const int D = s.cfg.dim;
  auto O = [&](int q) -> double& { return out[(size_t)q * n + a]; };
  for (int k = 0; k < 3; k++) {
    O(SF_R + k) = k < D ? s.r[k][a] : 0.0;
    O(SF_U + k) = k < D ? s.u[k][a] : 0.0;
    O(SF_GP + k) = k < D ? s.gradP[k][a] : 0.0;
    O(SF_GE + k) = k < D ? s.gradE[k][a] : 0.0;
  }
  O(SF_S) = s.th[kS][a];
  O(SF_E) = s.th[kE][a];
  O(SF_RB) = s.th[kRhoB][a];
  O(SF_RS) = s.th[kRhoS][a];
  O(SF_RQ) = s.th[kRhoQ][a];
  O(SF_T) = s.th[kT][a];
  O(SF_MUB) = s.th[kMuB][a];
  O(SF_MUS) = s.th[kMuS][a];
  O(SF_MUQ) = s.th[kMuQ][a];
  O(SF_THETA) = s.theta[a];
  O(SF_BULK) = s.bulk[a];
  O(SF_SLAB) = s.sigma_lab[a];
  const int sl[10][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {1, 1}, {1, 2}, {1, 3}, {2, 2}, {2, 3}, {3, 3}};
  for (int q = 0; q < 10; q++) O(SF_SHV + q) = s.shv[sl[q][0] * 4 + sl[q][1]][a];
  O(SF_SHV33) = s.shv[15][a];
  O(SF_SNU) = s.shv_nabla_u[a];
  O(SF_W) = s.th[kW][a];
  O(SF_CS2) = s.th[kCs2][a];
  for (int k = 0; k < 12; k++) O(SF_Q + k) = s.q[k][a];
}

void copy_snapshot(std::vector<double>& dst, const std::vector<double>& src, int a, int n) {
  for (int q = 0; q < NSF; q++) dst[(size_t)q * n + a] = src[(size_t)q * n + a];
}

// bsqsvinterpolate for particle a (status 3), from snapshot S taken at tp
void interpolate(System& s, int a, const std::vector<double>& Sv, double tp) {
  const int D = s.cfg.dim, n = s.n;
  auto S = [&](int q) { return Sv[(size_t)q * n + a]; };
  const double tlist = s.btrack[a] != -1 ? tp : tp - s.cfg.dt;
  const double t2 = tlist * tlist;
  double uout[3], ucov[3], gP[3], gE[3], gPc[3], gEc[3];
  for (int k = 0; k < D; k++) {
    uout[k] = S(SF_U + k);
    gP[k] = S(SF_GP + k);
    gE[k] = S(SF_GE + k);
    ucov[k] = -uout[k];
    gPc[k] = -gP[k];
    gEc[k] = -gE[k];
  }
  if (s.cfg.coord == 0 && D == 3) {   // milne::Vector make_covariant / make_contravariant
    ucov[2] = uout[2] * -t2;
    gPc[2] = gP[2] * (-1. / t2);
    gEc[2] = gE[2] * (-1. / t2);
  }
  const double bulk = S(SF_BULK), theta = S(SF_THETA), snu = S(SF_SNU);
  double sigsub = S(SF_SLAB);
  const double Efluc = S(SF_E);
  double Tfluc = S(SF_T), sFO = S(SF_S);
  double norm2 = 0.0;
  for (int k = 0; k < D; k++) norm2 += uout[k] * ucov[k];
  const double gsub = std::sqrt(-norm2 + 1);
  if (s.cfg.coord == 1) sigsub /= gsub;
  else sigsub /= gsub * tlist;
  const double swsub = s.mass[0][a] / sigsub;
  double divT[3], divE[3], divTc[3];
  for (int k = 0; k < D; k++) {
    divT[k] = (1.0 / sFO) * gP[k];
    divE[k] = gE[k];
    divTc[k] = (1.0 / sFO) * gPc[k];
  }
  const double cs2 = S(SF_CS2), w = S(SF_W);
  double inner = 0;
  for (int k = 0; k < D; k++) inner += uout[k] * gP[k];
  const double divPpress = -(1.0 / gsub) * (cs2 * (w + bulk) * theta - cs2 * snu + inner);
  double divTtemp = divPpress / sFO;
  inner = 0;
  for (int k = 0; k < D; k++) inner += uout[k] * gE[k];
  double divEener = -(1.0 / gsub) * ((w + bulk) * theta - snu + inner);
  norm2 = 0;
  for (int k = 0; k < D; k++) norm2 += divT[k] * divTc[k];
  const double insub = divTtemp * divTtemp + norm2;
  double nrm = -std::sqrt(std::fabs(insub));
  nrm = std::fabs(nrm) > 1.E-14 ? nrm : 1.E-14;
  divTtemp /= nrm;
  for (int k = 0; k < D; k++) divT[k] /= nrm;
  norm2 = 0;
  for (int k = 0; k < D; k++) norm2 += divE[k] * gEc[k];
  const double insubE = divEener * divEener + norm2;
  double nrmE = -std::sqrt(std::fabs(insubE));
  nrmE = std::fabs(nrmE) > 1.E-14 ? nrmE : 1.E-14;
  divEener /= nrmE;
  for (int k = 0; k < D; k++) divE[k] /= nrmE;
  sFO *= std::pow(Tfluc * 0.1973269804, 3);
  Tfluc *= 0.1973269804;
  // the row of freeze_out.dat (src/output.cpp:433-475)
  std::vector<double> row = {(double)s.nstep, (double)a, divEener};
  for (int k = 0; k < D; k++) row.push_back(divE[k]);
  row.push_back(gsub);
  for (int k = 0; k < D; k++) row.push_back(uout[k]);
  row.push_back(swsub);
  row.push_back(bulk);
  row.push_back(S(SF_SHV + 0));   // (0,0)
  row.push_back(S(SF_SHV + 4));   // (1,1)
  row.push_back(S(SF_SHV + 7));   // (2,2)
  row.push_back(S(SF_SHV33));
  row.push_back(S(SF_SHV + 5));   // (1,2)
  if (D != 2) {
    row.push_back(S(SF_SHV + 6));  // (1,3)
    row.push_back(S(SF_SHV + 8));  // (2,3)
  }
  row.push_back(tlist);
  for (int k = 0; k < D; k++) row.push_back(S(SF_R + k));
  for (double v : {sFO, Efluc, Tfluc, S(SF_MUB), S(SF_MUS), S(SF_MUQ), S(SF_W), cs2, S(SF_RB), S(SF_RS), S(SF_RQ)})
    row.push_back(v);
  for (int k = 0; k < 12; k++) row.push_back(S(SF_Q + k));   // q^mu of the snapshot (diffout)
  row.push_back(s.eos_id[a] >= 0 && s.cfg.eos_kind == 2 && s.eos_id[a] == 0 ? 1.0 : 0.0);
  s.fo_rows.push_back(row);
}

}  // namespace

void freeze_out_status(System& s) {
  const double ef = s.efcheck;
  const int frzc = s.frzc, n = s.n;
  const bool surf = s.cfg.surface != 0;
  if ((int)s.frz1_e.size() != n) s.frz1_e.assign(n, 0.0);
  if (surf && (int)s.snap[0].size() != NSF * n)
    for (int k = 0; k < 6; k++) s.snap[k].assign((size_t)NSF * n, 0.0);
  std::vector<double>&frz1 = s.snap[0], &frz2 = s.snap[1], &fb1 = s.snap[2], &fb2 = s.snap[3], &fb3 = s.snap[4],
      &fb4 = s.snap[5];
  const double t = s.t;
  // times of the snapshots as the interpolation sees them (the second step
  // sets taup before interpolating)
  const double taup = frzc == 1 ? t : s.taup, taupp = s.taupp;
  std::vector<double> cur;
  if (surf) cur.assign((size_t)NSF * n, 0.0);
  for (int a = 0; a < n; a++) {
    // check_freeze_out_status
    int f = s.freeze[a];
    const double e = s.th[kE][a];
    if (f == 0) {
      if (e <= ef) f = 1;
    } else if (f == 1) {
      if (s.btrack[a] == -1) f = 3;
      else if (e > s.frz1_e[a]) f = 1;
      else if (e <= ef) f = 3;
      else f = 0;
    }
    if (surf) take_snapshot(s, a, cur.data(), n);
    // bsqsvfreezeout
    if (frzc == 0) {
      if (surf) copy_snapshot(frz2, cur, a, n);
    } else if (frzc == 1) {
      s.frz1_e[a] = e;
      if (surf) copy_snapshot(frz1, cur, a, n);
      if (f == 3) {
        if (surf) {
          const double d1 = std::fabs(frz1[(size_t)SF_E * n + a] - ef), d2 = std::fabs(frz2[(size_t)SF_E * n + a] - ef);
          interpolate(s, a, d1 < d2 ? frz1 : frz2, d1 < d2 ? taup : taupp);
        }
        f = 4;
      }
    } else {
      const int bt = s.btrack[a];
      if (surf) {
        if (f < 4 && bt <= 3 && bt > 0) {
          copy_snapshot(fb4, fb2, a, n);
          copy_snapshot(fb3, fb1, a, n);
          copy_snapshot(fb2, frz2, a, n);
          copy_snapshot(fb1, frz1, a, n);
        }
        if (f < 4 && bt == 0 && fb1[(size_t)SF_GP * n + a] != 0) {
          copy_snapshot(frz2, fb2, a, n);
          copy_snapshot(frz1, fb1, a, n);
        }
        if (f < 4 && bt == 0 && fb1[(size_t)SF_GP * n + a] == 0) {
          copy_snapshot(frz2, fb4, a, n);
          copy_snapshot(frz1, fb3, a, n);
        }
      }
      if (f < 4 && bt == 0) {
        f = 4;
        s.btrack[a] = -1;
      }
      if (f == 3) {
        if (surf) {
          const double d1 = std::fabs(frz1[(size_t)SF_E * n + a] - ef), d2 = std::fabs(frz2[(size_t)SF_E * n + a] - ef);
          interpolate(s, a, d1 < d2 ? frz1 : frz2, d1 < d2 ? taup : taupp);
        }
        f = 4;
      }
      if (surf) {
        if (f < 4) copy_snapshot(frz2, frz1, a, n);
        copy_snapshot(frz1, cur, a, n);
      }
      if (f < 4) s.frz1_e[a] = e;
    }
    s.freeze[a] = f;
  }
  if (frzc == 0) s.taupp = t;
  else if (frzc == 1) s.taup = t;
  else {
    s.taupp = s.taup;
    s.taup = t;
  }
  s.frzc = frzc < 2 ? frzc + 1 : 2;
  s.nstep++;
}

// src/system_state.cpp:738-885 (entropy, BSQ, energy totals), with the
// diffusion q^0 terms when the diffusion sector is on.
Totals conservation(const System& s) {
  Totals T{0, 0, 0, 0, 0, 0};
  const double sqrtg = s.cfg.coord == 0 ? s.t : 1.0;
  for (int a = 0; a < s.n; a++) {
    const double g = s.gamma[a];
    T.S += s.ext[0][a] * s.mass[0][a];
    if (s.cfg.using_diffusion) {
      // the q^0 terms of :755-828, each with the reference's mass factors
      const double sg = s.sigma[a];
      const double eqb = s.q[0][a] * s.mass[1][a] / sg / g;
      const double eqs = s.q[4][a] * s.mass[0][a] / sg / g;
      const double eqq = s.q[8][a] * s.mass[0][a] / sg / g;
      T.B += s.ext[1][a] * s.mass[1][a] + eqb * s.mass[1][a] / g;
      T.Sq += s.ext[2][a] * s.mass[2][a] + (eqs);
      T.Q += s.ext[3][a] * s.mass[3][a] + (eqq);
    } else {
      T.B += s.ext[1][a] * s.mass[1][a];
      T.Sq += s.ext[2][a] * s.mass[2][a];
      T.Q += s.ext[3][a] * s.mass[3][a];
    }
    const double C = s.th[kW][a] + s.bulk[a];
    T.E += (C * g * g - s.th[kP][a] - s.bulk[a] + s.shv[0][a]) * s.mass[0][a] * sqrtg / s.sigma_lab[a];
    T.Ez += s.Ez[a];
  }
  return T;
}

// src/BSQHydro.cpp:568-646 (initialize_hydrodynamics) with
// src/sph_workstation.cpp:1228-1340 (process_initial_conditions),
// :252-375 (initialize_entropy_and_charge_densities) and :394-457
// (initial_smoothing); no freeze-in, sources or jets.
int initialize(System& s, NbrList& nl) {
  const int D = s.cfg.dim;
  s.t = s.cfg.t0;
  const double tm = s.cfg.coord == 1 ? 1.0 : s.t, t2 = tm * tm;
  const double T_seed = 580.0 / kHbarcMeVfm;
  for (int a = 0; a < s.n; a++) {
    double u[3] = {s.u[0][a], s.u[1][a], s.u[2][a]};
    s.gamma[a] = gamma_of(D, u, t2);
    for (int k = 0; k < 4; k++) { s.ext[k][a] = 1.0; s.mass[k][a] = 1.0; }
    s.th[kT][a] = T_seed;
    s.th[kMuB][a] = s.th[kMuS][a] = s.th[kMuQ][a] = 0.0;
    s.eos_id[a] = 0;
    s.freeze[a] = 0;
    s.btrack[a] = 0;
    s.Ez[a] = 0.0;
  }
  build_neighbours(s, nl);
  // freeze-out energy density: e(T_FO, 0, 0, 0) of the default EoS
  double efc = 0;
  {
    double x[4] = {s.cfg.freeze_out_T, 0, 0, 0}, o[17];
    eos_full_thermo(s.cfg, s.table, 0, x, o);
    efc = o[5];
  }
  s.efcheck = efc;
  s.frzc = 0;
  s.frz1_e.assign(s.n, 0.0);
  int bad = 0;
#pragma omp parallel for reduction(+ : bad)
  for (int a = 0; a < s.n; a++) {
    double x[4] = {s.th[kT][a], 0, 0, 0};
    int it = 0, k;
    if (s.cfg.input_as_entropy) {
      double tgt[4] = {s.in_s[a], s.in_rho[0][a], s.in_rho[1][a], s.in_rho[2][a]};
      k = eos_invert(s.cfg, s.table, 1, tgt, 0, x, &it);
    } else {
      double tgt[4] = {s.in_e[a], s.in_rho[0][a], s.in_rho[1][a], s.in_rho[2][a]};
      k = eos_invert(s.cfg, s.table, 0, tgt, 0, x, &it);
      if (k < 0) {
        s.freeze[a] = 4;
        double tz[4] = {s.in_e[a], 0, 0, 0};
        x[0] = s.th[kT][a]; x[1] = x[2] = x[3] = 0;
        k = eos_invert(s.cfg, s.table, 0, tz, 0, x, &it);
      }
    }
    if (k < 0) { s.eos_status[a] = -1; s.eos_id[a] = -1; bad++; continue; }
    double th[16];
    eos_set_thermo(s.cfg, s.table, k, x, th);
    for (int j = 0; j < 16; j++) s.th[j][a] = th[j];
    s.eos_id[a] = k;
    s.eos_status[a] = it;
    if (s.cfg.input_as_entropy) s.in_e[a] = th[kE]; else s.in_s[a] = th[kS];
    if (!(s.in_e[a] > efc && s.freeze[a] != 4)) s.freeze[a] = 4;
  }
  // no solution even at zero charge: the reference throws here
  // (src/sph_workstation.cpp:1840-1846); the count is returned instead
  if (bad) return bad;
  calculate_initial_sigma(s, nl, s.cfg.t0);
  for (int a = 0; a < s.n; a++) {
    const double sg = s.sigma[a];
    for (int k = 0; k < 4; k++) s.mass[k][a] = 1;
    s.ext[0][a] = s.in_s[a] / sg;
    for (int k = 1; k < 4; k++) s.ext[k][a] = s.in_rho[k - 1][a] / sg;
    if (s.in_s[a] < 0.0) s.freeze[a] = 4;
  }
  update_velocity(s);
  // initial_smoothing
  update_velocity(s);
  smooth_fields(s, nl);
  // calculate_extensive_shv and set_bulk_Pi (src/sph_workstation.cpp:
  // 1350-1430): the input pi^{ij} / sigma with input_initial_shear, (trace -
  // p) / sigma with bulk_from_trace (p of the e -> s inversion), else zero
  for (int a = 0; a < s.n; a++) {
    for (int k = 0; k < 6; k++) s.ext_shv[k][a] = (s.use_in_shv && k < 5) ? s.in_shv[k][a] / s.sigma[a] : 0.0;
    for (int k = 0; k < 16; k++) s.shv[k][a] = 0.0;
    s.ext_bulk[a] = s.use_in_bulk ? (s.in_bulk[a] - s.th[kP][a]) / s.sigma[a] : 0.0;
    s.bulk[a] = 0.0;
    // set_diffusion (src/sph_workstation.cpp:1441-1458): ext q = q^i / sigma
    for (int c = 0; c < 3; c++)
      for (int i = 0; i < 3; i++)
        s.ext_q[3 * c + i][a] = s.cfg.using_diffusion ? s.in_q[4 * c + i + 1][a] / s.sigma[a] : 0.0;
  }
  reset_pi_tensor(s);
  update_thermodynamics(s);
  return 0;
}

}  // namespace orc
