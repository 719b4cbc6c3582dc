// On-disk formats of the reference, host side: the "ccake" initial-condition
// text format (reader) and the system_state_N.dat text output (writer).
//
// Reader: src/BSQHydro.cpp:206-425 (read_ccake). One header line
// "#<ignored> dx dy deta <ignored> xmin ymin etamin", then one cell a line:
//   x y eta e|s rhoB rhoS rhoQ ux uy ueta bulk pixx pixy pixeta piyy piyeta pietaeta
// and, with initial diffusion, 12 more: qB^0..3 qS^0..3 qQ^0..3. Blank lines
// and '#' lines after the header are skipped; e (GeV/fm^3), the pi^{ij} and
// the bulk pressure are divided by hbar c; disabled charges read as zero;
// cells at or below e_cutoff are dropped (with entropy input, by the ideal
// pion-gas energy of s).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "ccake_gpu.h"
#include "common.cuh"

using namespace ccake;

struct ccake_ic {
  double grid[6] = {0, 0, 0, 0, 0, 0};   // dx, dy, deta, xmin, ymin, etamin
  std::string header;
  // columns in file order (17 + 12 diffusion), internal units
  std::vector<double> col[29];
  int64_t n = 0;
};

namespace {

const char* const kIcColumns[29] = {"x",    "y",    "eta",    "e",     "rhoB",   "rhoS",     "rhoQ", "ux",
                                    "uy",   "ueta", "bulk",   "pixx",  "pixy",   "pixeta",   "piyy", "piyeta",
                                    "pietaeta", "qB0", "qB1", "qB2",  "qB3",    "qS0",      "qS1",  "qS2",
                                    "qS3",  "qQ0",  "qQ1",    "qQ2",   "qQ3"};

int ic_column_index(const char* name) {
  if (std::strcmp(name, "s") == 0) return 3;   // the same column under entropy input
  for (int k = 0; k < 29; k++)
    if (std::strcmp(name, kIcColumns[k]) == 0) return k;
  return -1;
}

}  // namespace

extern "C" {

ccake_status_t ccake_ic_read_ccake(const char* path, const ccake_ic_options* opt, ccake_ic** out) {
  if (!path || !opt || !out) return CCAKE_ERR_INVALID;
  *out = nullptr;
  std::ifstream in(path);
  if (!in.is_open()) return CCAKE_ERR_INVALID;
  std::unique_ptr<ccake_ic> ic(new (std::nothrow) ccake_ic());
  if (!ic) return CCAKE_ERR_NOMEM;
  std::string line;
  if (!std::getline(in, line)) return CCAKE_ERR_INVALID;
  ic->header = line;
  {
    // text after the first '#': ignored, dx, dy, deta, ignored, xmin, ymin, etamin
    const size_t h = line.find('#');
    if (h == std::string::npos) return CCAKE_ERR_INVALID;
    std::istringstream hs(line.substr(h + 1));
    double ign0, ign1;
    if (!(hs >> ign0 >> ic->grid[0] >> ic->grid[1] >> ic->grid[2] >> ign1 >> ic->grid[3] >> ic->grid[4] >> ic->grid[5]))
      return CCAKE_ERR_INVALID;
  }
  const int ncol = opt->input_initial_diffusion ? 29 : 17;
  const double ecut = opt->e_cutoff / kHbarcGeVfm;
  // C = g_pi pi^2 / 90 of the ideal pion gas, e(s) = 3C (s / 4C)^{4/3}
  const double C = 3.0 * M_PI * M_PI / 90.0;
  const double eps_of_s = (3.0 * C) * std::pow(1.0 / (4.0 * C), 4.0 / 3.0);
  const bool charge[3] = {opt->baryon != 0, opt->strange != 0, opt->electric != 0};
  double v[29];
  while (std::getline(in, line)) {
    const size_t nb = line.find_first_not_of(" \t\r\n");
    if (nb == std::string::npos || line[nb] == '#') continue;
    std::istringstream ls(line);
    for (int k = 0; k < ncol; k++)
      if (!(ls >> v[k])) return CCAKE_ERR_INVALID;   // a short data line
    for (int k = ncol; k < 29; k++) v[k] = 0.0;
    if (!opt->input_as_entropy) v[3] /= kHbarcGeVfm;                 // e: GeV/fm^3 -> 1/fm^4
    for (int k = 10; k < 17; k++) v[k] /= kHbarcGeVfm;               // bulk, pi^{ij}
    for (int c = 0; c < 3; c++)
      if (!charge[c]) {
        v[4 + c] = 0.0;
        for (int m = 0; m < 4; m++) v[17 + 4 * c + m] = 0.0;
      }
    const double e_check = opt->input_as_entropy ? eps_of_s * std::pow(v[3], 4.0 / 3.0) : v[3];
    if (!(e_check > ecut)) continue;
    for (int k = 0; k < 29; k++) ic->col[k].push_back(v[k]);
    ic->n++;
  }
  *out = ic.release();
  return CCAKE_OK;
}

ccake_status_t ccake_ic_info(const ccake_ic* ic, int64_t* n, double* grid6) {
  if (!ic || !n) return CCAKE_ERR_INVALID;
  *n = ic->n;
  if (grid6)
    for (int k = 0; k < 6; k++) grid6[k] = ic->grid[k];
  return CCAKE_OK;
}

ccake_status_t ccake_ic_column(const ccake_ic* ic, const char* name, double* dst) {
  if (!ic || !name || (!dst && ic->n > 0)) return CCAKE_ERR_INVALID;
  const int k = ic_column_index(name);
  if (k < 0) return CCAKE_ERR_INVALID;
  if (ic->n > 0) std::memcpy(dst, ic->col[k].data(), (size_t)ic->n * sizeof(double));
  return CCAKE_OK;
}

ccake_status_t ccake_ic_particles(const ccake_ic* ic, ccake_particles_soa* soa) {
  if (!ic || !soa) return CCAKE_ERR_INVALID;
  soa->n = ic->n;
  soa->x = ic->col[0].data();
  soa->y = ic->col[1].data();
  soa->eta = ic->col[2].data();
  soa->e_or_s = ic->col[3].data();
  soa->rhoB = ic->col[4].data();
  soa->rhoS = ic->col[5].data();
  soa->rhoQ = ic->col[6].data();
  soa->ux = ic->col[7].data();
  soa->uy = ic->col[8].data();
  soa->ueta = ic->col[9].data();
  return CCAKE_OK;
}

void ccake_ic_free(ccake_ic* ic) { delete ic; }

}  // extern "C"
