// CPU oracle: SPH kernel, neighbour search, field smoothing, gradient sums.
// TEST INFRASTRUCTURE ONLY (see oracle.hpp).
#include "oracle.hpp"

#include <algorithm>
#include <cmath>
#include <unordered_map>

namespace orc {

namespace {
// Kernel normalisations, src/kernel.cpp:11-26.
double knorm(int D) { return D == 1 ? 2. / 3. : D == 2 ? 10. / (7 * M_PI) : 1. / M_PI; }
double knorm2(int D) { return D == 1 ? 1. / 6. : D == 2 ? 5. / (14. * M_PI) : 1. / (4 * M_PI); }
double kgrad(int D) { return D == 1 ? -1. / 2. : D == 2 ? -15. / (14. * M_PI) : -3. / (4. * M_PI); }
double kgrad2(int D) { return D == 1 ? 1. : D == 2 ? 15. / (7. * M_PI) : 3. / (2. * M_PI); }
}  // namespace

// Cubic spline W(q), q = r/h, support 2h. src/kernel.cpp:34-48.
double kernel_W(int D, double r, double h) {
  double norm = knorm(D) / std::pow(h, D);
  double norm2 = knorm2(D) / std::pow(h, D);
  double q = r / h;
  if (q >= 2.0) return 0.0;
  if (q >= 1.0) return norm2 * (2.0 - q) * (2.0 - q) * (2.0 - q);
  double qq = q * q;
  return norm * (1 - 1.5 * qq + 0.75 * q * qq);
}

// Gradient of W with respect to r_a, rel = r_a - r_b. src/kernel.cpp:95-118.
void kernel_gradW(int D, const double* rel, double r, double h, double* grad) {
  double ng = kgrad(D) / std::pow(h, D + 1);
  double ng2 = kgrad2(D) / std::pow(h, D + 1);
  double q = r / h;
  if (q >= 2.0) {
    for (int i = 0; i < D; i++) grad[i] = 0.0;
    return;
  }
  if (q >= 1.0) {
    for (int i = 0; i < D; i++) grad[i] = (ng / r) * (2.0 - q) * (2.0 - q) * rel[i];
    return;
  }
  for (int i = 0; i < D; i++) grad[i] = ng2 * (1.5 * q - 2) * rel[i] / h;
}

// Factorised 3-D kernel W2D(r_perp,hT)*W1D(|deta|,hEta). src/kernel.cpp:130-138.
double kernel_W_factorized(const double* r1, const double* r2, double hT, double hEta) {
  double dx = r1[0] - r2[0], dy = r1[1] - r2[1];
  double rp = std::sqrt(dx * dx + dy * dy);
  double de = std::sqrt((r1[2] - r2[2]) * (r1[2] - r2[2]));
  return kernel_W(2, rp, hT) * kernel_W(1, de, hEta);
}

// src/kernel.cpp:152-170.
void kernel_gradW_factorized(const double* rel, double hT, double hEta, double* grad) {
  double rp = std::sqrt(rel[0] * rel[0] + rel[1] * rel[1]);
  double de = std::sqrt(rel[2] * rel[2]);
  double g2[2], g1;
  kernel_gradW(2, rel, rp, hT, g2);
  kernel_gradW(1, &rel[2], de, hEta, &g1);
  double W2 = kernel_W(2, rp, hT), W1 = kernel_W(1, de, hEta);
  grad[0] = g2[0] * W1;
  grad[1] = g2[1] * W1;
  grad[2] = W2 * g1;
}

// Neighbour predicate of the reference's Cabana VerletList (full list, cutoff
// 2h, call site src/system_state.cpp:698-700): squared distance over the three
// position components (unused components are zero) compared with <= (2h)^2.
// Evaluated without fused multiply-add (the oracle is built -ffp-contract=off).
static inline bool within(const System& s, int a, int b, double rsqr) {
  double dx = s.r[0][a] - s.r[0][b];
  double dy = s.r[1][a] - s.r[1][b];
  double dz = s.r[2][a] - s.r[2][b];
  double d2 = dx * dx + dy * dy + dz * dz;
  return d2 <= rsqr;
}

void neighbours_bruteforce(const System& s, std::vector<int32_t>& off, std::vector<int32_t>& idx) {
  double cut = 2 * s.cfg.hT, rsqr = cut * cut;
  off.assign(s.n + 1, 0);
  idx.clear();
  for (int a = 0; a < s.n; a++) {
    for (int b = 0; b < s.n; b++)
      if (b != a && within(s, a, b, rsqr)) idx.push_back(b);
    off[a + 1] = (int32_t)idx.size();
  }
}

void neighbours_celllist(const System& s, std::vector<int32_t>& off, std::vector<int32_t>& idx) {
  const double cut = 2 * s.cfg.hT, rsqr = cut * cut;
  double lo[3] = {1e300, 1e300, 1e300};
  for (int d = 0; d < 3; d++)
    for (int i = 0; i < s.n; i++) lo[d] = std::min(lo[d], s.r[d][i]);
  auto cell = [&](int i, int d) { return (int64_t)std::floor((s.r[d][i] - lo[d]) / cut); };
  auto key = [](int64_t x, int64_t y, int64_t z) { return (x * 1000003LL + y) * 1000033LL + z; };
  std::unordered_map<int64_t, std::vector<int32_t>> grid;
  for (int i = 0; i < s.n; i++) grid[key(cell(i, 0), cell(i, 1), cell(i, 2))].push_back(i);
  std::vector<std::vector<int32_t>> lists(s.n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int a = 0; a < s.n; a++) {
    int64_t cx = cell(a, 0), cy = cell(a, 1), cz = cell(a, 2);
    auto& L = lists[a];
    for (int64_t ix = cx - 1; ix <= cx + 1; ix++)
      for (int64_t iy = cy - 1; iy <= cy + 1; iy++)
        for (int64_t iz = cz - 1; iz <= cz + 1; iz++) {
          auto it = grid.find(key(ix, iy, iz));
          if (it == grid.end()) continue;
          for (int32_t b : it->second)
            if (b != a && within(s, a, b, rsqr)) L.push_back(b);
        }
    std::sort(L.begin(), L.end());
  }
  off.assign(s.n + 1, 0);
  for (int a = 0; a < s.n; a++) off[a + 1] = off[a] + (int32_t)lists[a].size();
  idx.resize(off[s.n]);
  for (int a = 0; a < s.n; a++) std::copy(lists[a].begin(), lists[a].end(), idx.begin() + off[a]);
}

// src/system_state.cpp:650-719 (list rebuilt from current positions; btrack =
// number of neighbours).
void build_neighbours(System& s, NbrList& nl) {
  if (s.n <= 2048)
    neighbours_bruteforce(s, nl.off, nl.idx);
  else
    neighbours_celllist(s, nl.off, nl.idx);
  for (int a = 0; a < s.n; a++)
    s.btrack[a] = (s.btrack[a] == -1) ? -1 : nl.off[a + 1] - nl.off[a];
}

static inline double pair_W(const System& s, int a, int b) {
  const int D = s.cfg.dim;
  double r1[3], r2[3];
  for (int d = 0; d < D; d++) { r1[d] = s.r[d][a]; r2[d] = s.r[d][b]; }
  if (D == 3 && s.cfg.factorized_kernel) return kernel_W_factorized(r1, r2, s.cfg.hT, s.cfg.hEta);
  double d2 = 0;
  for (int d = 0; d < D; d++) { double x = r1[d] - r2[d]; d2 += x * x; }
  return kernel_W(D, std::sqrt(d2), s.cfg.hT);
}

static inline double kern0(const System& s) {
  const int D = s.cfg.dim;
  if (D == 3 && s.cfg.factorized_kernel) {
    double z[3] = {0, 0, 0};
    return kernel_W_factorized(z, z, s.cfg.hT, s.cfg.hEta);
  }
  return kernel_W(D, 0.0, s.cfg.hT);
}

// Lab-frame to local-rest-frame factor: Milne lab/(gamma*t)
// (src/eom_default.cpp:198-203); Cartesian lab/gamma (src/eom_cartesian.cpp:196-201).
static inline double lrf(const System& s, double lab, double gamma, double t) {
  return s.cfg.coord == 0 ? lab / gamma / t : lab / gamma;
}

// src/sph_workstation.cpp:494-578 (smooth_all_particle_fields).
void smooth_fields(System& s, const NbrList& nl) {
  const double k0 = kern0(s);
  const double t = s.t;
#pragma omp parallel for schedule(static)
  for (int a = 0; a < s.n; a++) {
    double sm[4], slab = s.mass[0][a] * k0;
    for (int k = 0; k < 4; k++) sm[k] = s.mass[k][a] * s.ext[k][a] * k0;
    for (int j = nl.off[a]; j < nl.off[a + 1]; j++) {
      int b = nl.idx[j];
      double W = pair_W(s, a, b);
      slab += s.mass[0][b] * W;
      for (int k = 0; k < 4; k++) sm[k] += s.mass[k][b] * s.ext[k][b] * W;
    }
    for (int k = 0; k < 4; k++) s.smoothed[k][a] = sm[k];
    s.sigma_lab[a] = slab;
    double g = s.gamma[a];
    s.sigma[a] = lrf(s, slab, g, t);
    s.th[kS][a] = lrf(s, sm[0], g, t);
    s.th[kRhoB][a] = lrf(s, sm[1], g, t);
    s.th[kRhoS][a] = lrf(s, sm[2], g, t);
    s.th[kRhoQ][a] = lrf(s, sm[3], g, t);
  }
}

// src/sph_workstation.cpp:582-640 (calculate_intial_sigma).
void calculate_initial_sigma(System& s, const NbrList& nl, double t) {
  const double k0 = kern0(s);
#pragma omp parallel for schedule(static)
  for (int a = 0; a < s.n; a++) {
    double slab = s.mass[0][a] * k0;
    for (int j = nl.off[a]; j < nl.off[a + 1]; j++) slab += s.mass[0][nl.idx[j]] * pair_W(s, a, nl.idx[j]);
    s.sigma_lab[a] = slab;
    s.sigma[a] = lrf(s, slab, s.gamma[a], t);
  }
}

// src/sph_workstation.cpp:796-986 (smooth_all_particle_gradients, generic /
// Milne form, D > 1, with the diffusion sums of :909-967).
void smooth_gradients(System& s, const NbrList& nl) {
  const int D = s.cfg.dim;
  const bool shear = s.cfg.using_shear;
  const bool diff = s.cfg.using_diffusion;
  const double hT = s.cfg.hT, hEta = s.cfg.hEta;
  const bool fact = (D == 3) && s.cfg.factorized_kernel;
#pragma omp parallel for schedule(static)
  for (int a = 0; a < s.n; a++) {
    double gP[3] = {0, 0, 0}, gE[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gS[3] = {0, 0, 0},
           dS[3] = {0, 0, 0}, gV[9] = {0};
    // diffusion sector (:909-967): v.grad q^0_a, div q_a, grad (mu_a / T)
    double gq[3] = {0, 0, 0}, dq[3] = {0, 0, 0}, ga[9] = {0};
    double alpha_a[3] = {0, 0, 0};
    if (diff) {
      alpha_a[0] = s.th[kMuB][a] / s.th[kT][a];
      alpha_a[1] = s.th[kMuS][a] / s.th[kT][a];
      alpha_a[2] = s.th[kMuQ][a] / s.th[kT][a];
    }
    const double pa = s.th[kP][a], ea = s.th[kE][a], sla = s.sigma_lab[a];
    const double sqa = 1.0 / (sla * sla);
    const double Pia = s.bulk[a];
    double va[3];
    for (int d = 0; d < D; d++) va[d] = s.v[d][a];
    for (int j = nl.off[a]; j < nl.off[a + 1]; j++) {
      const int b = nl.idx[j];
      double rel[3], pa_[3], pb_[3], gK[3];
      for (int d = 0; d < D; d++) {
        pa_[d] = s.r[d][a];
        pb_[d] = s.r[d][b];
        rel[d] = pa_[d] - pb_[d];
      }
      if (fact) {
        kernel_gradW_factorized(rel, hT, hEta, gK);
      } else {
        double d2 = 0;
        for (int d = 0; d < D; d++) { double x = pa_[d] - pb_[d]; d2 += x * x; }
        kernel_gradW(D, rel, std::sqrt(d2), hT, gK);
      }
      const double pb = s.th[kP][b], eb = s.th[kE][b], slb = s.sigma_lab[b];
      const double sqb = 1.0 / (slb * slb);
      const double mb = s.mass[0][b];
      const double Pib = s.bulk[b];
      double ssK[3];
      for (int d = 0; d < D; d++) ssK[d] = mb * sla * gK[d];
      for (int d = 0; d < D; d++) {
        gP[d] += (sqb * pb + sqa * pa) * ssK[d];
        gE[d] += (mb / sla) * (eb - ea) * gK[d];
        gB[d] += (Pib / slb / slb + Pia / sla / sla) * ssK[d];
      }
      for (int i = 0; i < D; i++)
        for (int k = 0; k < D; k++) gV[i * D + k] += (mb / sla) * (s.v[k][b] - va[k]) * gK[i];
      if (shear) {
        double ssKv = 0;
        for (int d = 0; d < D; d++) ssKv += ssK[d] * va[d];
        for (int i = 0; i < D; i++) {
          gS[i] += ssKv * (sqb * s.shv[0 * 4 + i + 1][b] + sqa * s.shv[0 * 4 + i + 1][a]);
          double acc = 0;
          for (int k = 0; k < D; k++)
            acc += sqb * ssK[k] * s.shv[(i + 1) * 4 + k + 1][b] + sqa * ssK[k] * s.shv[(i + 1) * 4 + k + 1][a];
          dS[i] += acc;
        }
      }
      if (diff) {
        const double alpha_b[3] = {s.th[kMuB][b] / s.th[kT][b], s.th[kMuS][b] / s.th[kT][b],
                                   s.th[kMuQ][b] / s.th[kT][b]};
        double ssKv = 0;
        for (int d = 0; d < D; d++) ssKv += ssK[d] * va[d];
        for (int c = 0; c < 3; c++) {
          gq[c] += ssKv * (sqb * s.q[4 * c][b] + sqa * s.q[4 * c][a]);
          double acc = 0.0;
          for (int i = 0; i < D; i++) {
            acc += sqb * ssK[i] * s.q[4 * c + i + 1][b] + sqa * ssK[i] * s.q[4 * c + i + 1][a];
            ga[3 * i + c] += (mb / sla) * (alpha_b[c] - alpha_a[c]) * gK[i];
          }
          dq[c] += acc;
        }
      }
    }
    if (diff) {
      for (int c = 0; c < 3; c++) {
        s.grad_qa[c][a] = gq[c];
        s.div_qa[c][a] = dq[c];
      }
      for (int k = 0; k < 9; k++) s.grad_alpha[k][a] = ga[k];
    }
    for (int d = 0; d < D; d++) {
      s.gradP[d][a] = gP[d];
      s.gradE[d][a] = gE[d];
      s.gradBulk[d][a] = gB[d];
      s.gradshear[d][a] = gS[d];
      s.divshear[d][a] = dS[d];
    }
    for (int i = 0; i < D * D; i++) s.gradV[i][a] = gV[i];
  }
}

}  // namespace orc
