// C entry points of the CPU oracle, loaded by the tests and the benchmark's
// CPU-baseline leg through ctypes. TEST INFRASTRUCTURE ONLY (see oracle.hpp).
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.hpp"
#include "table_oracle.hpp"

#include <cstring>
#include <string>

using namespace orc;

namespace {
struct Handle {
  System s;
  NbrList nl;
};

void alloc(System& s, int n) {
  auto A = [n](std::vector<double>& v) { v.assign(n, 0.0); };
  for (int i = 0; i < 3; i++) { A(s.r[i]); A(s.u[i]); A(s.v[i]); A(s.r0[i]); A(s.u0[i]); A(s.gradP[i]);
    A(s.gradE[i]); A(s.gradBulk[i]); A(s.gradshear[i]); A(s.divshear[i]); A(s.du_dt[i]); A(s.in_rho[i]); }
  for (int i = 0; i < 4; i++) { A(s.ext[i]); A(s.mass[i]); A(s.smoothed[i]); A(s.d_ext[i]); A(s.ext0[i]); }
  for (int i = 0; i < 6; i++) { A(s.ext_shv[i]); A(s.in_shv[i]); A(s.d_ext_shv[i]); A(s.ext_shv0[i]); }
  for (int i = 0; i < 9; i++) A(s.gradV[i]);
  for (int i = 0; i < 16; i++) { A(s.th[i]); A(s.shv[i]); }
  A(s.ext_bulk); A(s.Ez); A(s.in_e); A(s.in_s); A(s.in_bulk); A(s.gamma); A(s.sigma_lab); A(s.sigma);
  A(s.bulk); A(s.eta_pi); A(s.tau_pi); A(s.zeta_Pi); A(s.tau_Pi); A(s.delta_PiPi); A(s.delta_pipi);
  A(s.lambda_piPi); A(s.lambda_Pipi); A(s.phi1); A(s.phi3); A(s.phi6); A(s.phi7); A(s.tau_pipi);
  A(s.d_ext_bulk); A(s.dEz); A(s.theta); A(s.shv_nabla_u); A(s.ext_bulk0); A(s.Ez0);
  for (int i = 0; i < 5; i++) A(s.sigma_t[i]);
  A(s.kn_shear); A(s.kn_bulk); A(s.ire_shear); A(s.ire_bulk);
  for (int i = 0; i < 9; i++) { A(s.ext_q[i]); A(s.ext_q0[i]); A(s.tau_q[i]); A(s.kappa_q[i]); A(s.grad_alpha[i]);
    A(s.d_ext_q[i]); }
  for (int i = 0; i < 12; i++) { A(s.q[i]); A(s.in_q[i]); A(s.dalpha[i]); }
  for (int i = 0; i < 3; i++) { A(s.div_qa[i]); A(s.grad_qa[i]); A(s.kn_diff[i]); A(s.ire_diff[i]); }
  s.freeze.assign(n, 0); s.btrack.assign(n, 0); s.eos_id.assign(n, 0); s.eos_status.assign(n, 0);
  s.n = n;
}

std::vector<double>* field(System& s, const std::string& k) {
  static const char* thn[16] = {"T", "muB", "muS", "muQ", "p", "s", "rhoB", "rhoS", "rhoQ", "e", "w", "cs2",
                                "dwds", "dwdB", "dwdS", "dwdQ"};
  for (int i = 0; i < 16; i++) if (k == thn[i]) return &s.th[i];
  const char* xyz[3] = {"x", "y", "eta"};
  for (int i = 0; i < 3; i++) if (k == xyz[i]) return &s.r[i];
  for (int i = 0; i < 3; i++) {
    std::string d = std::to_string(i);
    if (k == "u" + d) return &s.u[i];
    if (k == "v" + d) return &s.v[i];
    if (k == "gradP" + d) return &s.gradP[i];
    if (k == "gradE" + d) return &s.gradE[i];
    if (k == "gradBulk" + d) return &s.gradBulk[i];
    if (k == "gradshear" + d) return &s.gradshear[i];
    if (k == "divshear" + d) return &s.divshear[i];
    if (k == "du_dt" + d) return &s.du_dt[i];
  }
  const char* dn[4] = {"s", "B", "S", "Q"};
  for (int i = 0; i < 4; i++) {
    if (k == std::string("ext_") + dn[i]) return &s.ext[i];
    if (k == std::string("d_ext_") + dn[i]) return &s.d_ext[i];
    if (k == std::string("smoothed_") + dn[i]) return &s.smoothed[i];
    if (k == std::string("mass_") + dn[i]) return &s.mass[i];
  }
  for (int i = 0; i < 5; i++) {
    if (k == "ext_shv" + std::to_string(i)) return &s.ext_shv[i];
    if (k == "d_ext_shv" + std::to_string(i)) return &s.d_ext_shv[i];
  }
  for (int i = 0; i < 9; i++) if (k == "gradV" + std::to_string(i)) return &s.gradV[i];
  for (int i = 0; i < 16; i++) if (k == "shv" + std::to_string(i / 4) + std::to_string(i % 4)) return &s.shv[i];
  if (k == "in_e") return &s.in_e;
  if (k == "in_s") return &s.in_s;
  if (k == "in_rhoB") return &s.in_rho[0];
  if (k == "in_rhoS") return &s.in_rho[1];
  if (k == "in_rhoQ") return &s.in_rho[2];
  if (k == "in_bulk") return &s.in_bulk;
  for (int i = 0; i < 6; i++) if (k == "in_shv" + std::to_string(i)) return &s.in_shv[i];
  if (k == "ext_bulk") return &s.ext_bulk;
  if (k == "Ez") return &s.Ez;
  if (k == "dEz") return &s.dEz;
  if (k == "gamma") return &s.gamma;
  if (k == "sigma_lab") return &s.sigma_lab;
  if (k == "sigma") return &s.sigma;
  if (k == "bulk") return &s.bulk;
  if (k == "eta_pi") return &s.eta_pi;
  if (k == "tau_pi") return &s.tau_pi;
  if (k == "zeta_Pi") return &s.zeta_Pi;
  if (k == "tau_Pi") return &s.tau_Pi;
  if (k == "d_ext_bulk") return &s.d_ext_bulk;
  if (k == "theta") return &s.theta;
  if (k == "shv_nabla_u") return &s.shv_nabla_u;
  for (int i = 0; i < 5; i++) if (k == "sigma_tensor" + std::to_string(i)) return &s.sigma_t[i];
  if (k == "shear_knudsen") return &s.kn_shear;
  if (k == "bulk_knudsen") return &s.kn_bulk;
  if (k == "inverse_reynolds_shear") return &s.ire_shear;
  if (k == "inverse_reynolds_bulk") return &s.ire_bulk;
  // diffusion sector: charge letters B, S, Q; q{c}{mu}, ext_q{c}{i},
  // d_ext_q{c}{i}, in_q{c}{mu}, tau_q{c}{d}, kappa_q{c}{d}, grad_alpha{i}{c},
  // dalpha{k} (0..11), div_qa{c}, grad_qa{c}, kn_diff{c}, ire_diff{c}
  const char ch[3] = {'B', 'S', 'Q'};
  for (int c = 0; c < 3; c++) {
    const std::string C(1, ch[c]);
    for (int m = 0; m < 4; m++) {
      if (k == "q" + C + std::to_string(m)) return &s.q[4 * c + m];
      if (k == "in_q" + C + std::to_string(m)) return &s.in_q[4 * c + m];
    }
    for (int i = 0; i < 3; i++) {
      if (k == "ext_q" + C + std::to_string(i)) return &s.ext_q[3 * c + i];
      if (k == "d_ext_q" + C + std::to_string(i)) return &s.d_ext_q[3 * c + i];
      if (k == "grad_alpha" + std::to_string(i) + C) return &s.grad_alpha[3 * i + c];
      if (k == "tau_q" + C + std::string(1, ch[i])) return &s.tau_q[3 * c + i];
      if (k == "kappa_q" + C + std::string(1, ch[i])) return &s.kappa_q[3 * c + i];
    }
    if (k == "div_qa" + C) return &s.div_qa[c];
    if (k == "grad_qa" + C) return &s.grad_qa[c];
    if (k == "kn_diff" + C) return &s.kn_diff[c];
    if (k == "ire_diff" + C) return &s.ire_diff[c];
  }
  for (int j = 0; j < 12; j++) if (k == "dalpha" + std::to_string(j)) return &s.dalpha[j];
  return nullptr;
}
}  // namespace

extern "C" {

void* orc_create(const Config* cfg, int n, const double* x, const double* y, const double* eta,
                 const double* e_or_s, const double* rhoB, const double* rhoS, const double* rhoQ,
                 const double* ux, const double* uy, const double* ueta, void* table) {
  Handle* h = new Handle;
  h->s.cfg = *cfg;
  alloc(h->s, n);
  h->s.table = (Table*)table;
  for (int i = 0; i < n; i++) {
    h->s.r[0][i] = x[i];
    h->s.r[1][i] = y[i];
    h->s.r[2][i] = (cfg->dim == 3 && eta) ? eta[i] : 0.0;
    h->s.u[0][i] = ux[i];
    h->s.u[1][i] = uy[i];
    h->s.u[2][i] = (cfg->dim == 3 && ueta) ? ueta[i] : 0.0;
    if (cfg->input_as_entropy) h->s.in_s[i] = e_or_s[i]; else h->s.in_e[i] = e_or_s[i];
    h->s.in_rho[0][i] = rhoB ? rhoB[i] : 0.0;
    h->s.in_rho[1][i] = rhoS ? rhoS[i] : 0.0;
    h->s.in_rho[2][i] = rhoQ ? rhoQ[i] : 0.0;
  }
  h->s.t = cfg->t0;
  return h;
}

void orc_destroy(void* p) { delete (Handle*)p; }

int orc_initialize(void* p) {
  Handle* h = (Handle*)p;
  const int failed = initialize(h->s, h->nl);
  if (failed) return failed;
  int bad = 0;
  for (int a = 0; a < h->s.n; a++) bad += (h->s.eos_status[a] < 0);
  return bad;
}

int orc_step(void* p, int nsteps) {
  Handle* h = (Handle*)p;
  for (int k = 0; k < nsteps; k++) rk2_step(h->s, h->nl);
  int bad = 0;
  for (int a = 0; a < h->s.n; a++) bad += (h->s.eos_status[a] < 0);
  return bad;
}

// Runs one named phase of a derivative evaluation at the current state.
int orc_phase(void* p, const char* name) {
  Handle* h = (Handle*)p;
  std::string k(name);
  if (k == "neighbours") build_neighbours(h->s, h->nl);
  else if (k == "velocity") update_velocity(h->s);
  else if (k == "smooth_fields") smooth_fields(h->s, h->nl);
  else if (k == "thermo") return update_thermodynamics(h->s);
  else if (k == "reset_pi") reset_pi_tensor(h->s);
  else if (k == "regulate_diffusion") regulate_diffusion(h->s);
  else if (k == "viscosities") update_viscosities(h->s);
  else if (k == "gradients") smooth_gradients(h->s, h->nl);
  else if (k == "eom") evaluate_time_derivatives(h->s);
  else if (k == "derivatives") get_time_derivatives(h->s, h->nl);
  else return -1;
  return 0;
}

void orc_set_initial_viscous(void* p, int bulk, int shear) {
  ((Handle*)p)->s.use_in_bulk = bulk;
  ((Handle*)p)->s.use_in_shv = shear;
}

double orc_time(void* p) { return ((Handle*)p)->s.t; }
void orc_set_time(void* p, double t) { ((Handle*)p)->s.t = t; }

int orc_get(void* p, const char* name, double* out) {
  Handle* h = (Handle*)p;
  auto* f = field(h->s, name);
  if (!f) return -1;
  std::memcpy(out, f->data(), sizeof(double) * h->s.n);
  return 0;
}

int orc_set(void* p, const char* name, const double* in) {
  Handle* h = (Handle*)p;
  auto* f = field(h->s, name);
  if (!f) return -1;
  std::memcpy(f->data(), in, sizeof(double) * h->s.n);
  return 0;
}

int orc_get_int(void* p, const char* name, int32_t* out) {
  Handle* h = (Handle*)p;
  std::string k(name);
  const std::vector<int32_t>* v = nullptr;
  if (k == "btrack") v = &h->s.btrack;
  else if (k == "freeze") v = &h->s.freeze;
  else if (k == "eos_id") v = &h->s.eos_id;
  else if (k == "eos_status") v = &h->s.eos_status;
  if (!v) return -1;
  std::memcpy(out, v->data(), sizeof(int32_t) * h->s.n);
  return 0;
}

void orc_totals(void* p, double* out6) {
  Totals T = conservation(((Handle*)p)->s);
  out6[0] = T.S; out6[1] = T.B; out6[2] = T.Sq; out6[3] = T.Q; out6[4] = T.E; out6[5] = T.Ez;
}

// Neighbour list of the current positions (CSR); returns the entry count, or
// -count when idx_cap is too small.
long orc_neighbours(void* p, int32_t* off, int32_t* idx, long idx_cap) {
  Handle* h = (Handle*)p;
  build_neighbours(h->s, h->nl);
  long m = (long)h->nl.idx.size();
  std::memcpy(off, h->nl.off.data(), sizeof(int32_t) * (h->s.n + 1));
  if (m > idx_cap) return -m;
  std::memcpy(idx, h->nl.idx.data(), sizeof(int32_t) * m);
  return m;
}

double orc_kernel_W(int D, double r, double h) { return kernel_W(D, r, h); }
void orc_kernel_gradW(int D, const double* rel, double r, double h, double* out) { kernel_gradW(D, rel, r, h, out); }

void* orc_table_create(const int32_t* n, const double* lo, const double* d, const double* fields,
                       const double* conf5, const double* cdiag5) {
  Table* t = new Table;
  for (int k = 0; k < 4; k++) { t->n[k] = n[k]; t->lo[k] = lo[k]; t->d[k] = d[k]; }
  size_t N = (size_t)n[0] * n[1] * n[2] * n[3] * 17;
  t->f.assign(fields, fields + N);
  t->conf = {conf5[0], conf5[1], conf5[2], conf5[3], conf5[4]};
  t->cdiag = {cdiag5[0], cdiag5[1], cdiag5[2], cdiag5[3], cdiag5[4]};
  return t;
}
void orc_table_destroy(void* t) { delete (Table*)t; }

// OpenMP threads of the oracle's parallel loops (timing baselines).
void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
  (void)n;
#endif
}

// Interpolated fields (17) and the Jacobian (5 x 4) of s, rhoB, rhoS, rhoQ, e
// with respect to (T, muB, muQ, muS) at one point.
void orc_table_jacobian(void* t, const double* x, double* out17, double* jac20) {
  double jac[5][4];
  table_full_thermo(*(Table*)t, x, out17, jac);
  for (int f = 0; f < 5; f++)
    for (int j = 0; j < 4; j++) jac20[4 * f + j] = jac[f][j];
}

void orc_eos_full_thermo(const Config* c, void* tab, int chain_index, const double* tbqs, double* out17) {
  eos_full_thermo(*c, (Table*)tab, chain_index, tbqs, out17);
}

// Batch inversion: in4 rows (e|s, B, S, Q); seed rows (T, muB, muQ, muS) are
// overwritten with the solution; th16 rows receive the derived thermo.
// status: chain index used (>= 0) or -1; iters: solver iterations.
void orc_eos_invert_batch(const Config* c, void* tab, int entropy, long n, const double* in4, double* tbqs4,
                          double* th16, int32_t* status, int32_t* iters) {
#pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < n; i++) {
    int it = 0;
    int k = eos_invert(*c, (Table*)tab, entropy, in4 + 4 * i, 0, tbqs4 + 4 * i, &it);
    status[i] = k;
    if (iters) iters[i] = it;
    if (k >= 0 && th16) eos_set_thermo(*c, (Table*)tab, k, tbqs4 + 4 * i, th16 + 16 * i);
  }
}

void orc_eos_alpha_derivs(const Config* c, void* tab, int chain_index, long n, const double* tbqs, double* out12) {
#pragma omp parallel for
  for (long i = 0; i < n; i++) eos_alpha_derivs(*c, (const Table*)tab, chain_index, tbqs + 4 * i, out12 + 12 * i);
}

void orc_eos_set_thermo(const Config* c, void* tab, int chain_index, const double* tbqs, double* th16) {
  eos_set_thermo(*c, (Table*)tab, chain_index, tbqs, th16);
}


int orc_fo_count(void* hp) { return (int)((Handle*)hp)->s.fo_rows.size(); }
int orc_fo_width(void* hp) {
  const auto& r = ((Handle*)hp)->s.fo_rows;
  return r.empty() ? 0 : (int)r[0].size();
}
void orc_fo_rows(void* hp, double* out) {
  size_t k = 0;
  for (const auto& row : ((Handle*)hp)->s.fo_rows)
    for (double v : row) out[k++] = v;
}

}  // extern "C"
