// CPU oracle: the tabulated 4-D EoS with the reference's multilinear lookup.
// TEST INFRASTRUCTURE ONLY (see oracle.hpp).
#pragma once
#include <cmath>
#include <vector>

namespace orc {

// Uniform (T, muB, muQ, muS) grid, row-major with muS fastest
// (include/interpolatorND.h:132-138), 17 fields per node in the order
// p s B S Q e cs2 chiBB chiQQ chiSS chiBQ chiBS chiQS chiTB chiTQ chiTS chiTT
// (src/eos_table.cpp:31-35). Axes in fm^-1 and fields in fm units after the
// loader's rescaling (src/eos_table.cpp:36-100).
struct Table {
  int n[4];
  double lo[4], d[4];
  std::vector<double> f;  // n0*n1*n2*n3*17
  struct { double c, T0, muB0, muQ0, muS0; } conf, cdiag;  // fallback model scales
};

// src/interpolatorND.cpp:250-317 (evaluate): index = integer part of
// (x - min)/spacing via modf (truncation toward zero), the last cell is reused
// at the upper edge, and any index outside [0, n) returns the NaN fill value.
// jac (optional): derivatives of the interpolated s, rhoB, rhoS, rhoQ, e
// (fields 1..5) with respect to (T, muB, muQ, muS): the exact Jacobian of the
// multilinear interpolant inside the cell.
inline void table_full_thermo(const Table& t, const double* x, double* out, double (*jac)[4] = nullptr) {
  int ind[4];
  double fr[4], dfr[4];
  for (int k = 0; k < 4; k++) {
    if (std::isnan(x[k])) { for (int i = 0; i < 17; i++) out[i] = NAN; return; }
    if (t.n[k] <= 1 || std::fabs(t.d[k]) < 1e-30) { ind[k] = 0; fr[k] = 1.0; dfr[k] = 0.0; continue; }
    double ip = 0.0;
    fr[k] = 1.0 - std::modf((x[k] - t.lo[k]) / t.d[k], &ip);
    dfr[k] = -1.0 / t.d[k];
    ind[k] = (int)ip;
    if (ind[k] + 1 == t.n[k]) { fr[k] = 1.0 - fr[k]; dfr[k] = -dfr[k]; ind[k]--; }
    if (ind[k] < 0 || ind[k] >= t.n[k]) { for (int i = 0; i < 17; i++) out[i] = NAN; return; }
  }
  for (int i = 0; i < 17; i++) out[i] = 0.0;
  if (jac)
    for (int f = 0; f < 5; f++) for (int j = 0; j < 4; j++) jac[f][j] = 0.0;
  for (int h = 0; h < 16; h++) {
    // hypercube corner bits, first axis is the most significant bit
    int b[4] = {(h >> 3) & 1, (h >> 2) & 1, (h >> 1) & 1, h & 1};
    double wk[4], w = 1.0;
    for (int k = 0; k < 4; k++) { wk[k] = fr[k] + b[k] - 2.0 * b[k] * fr[k]; w *= wk[k]; }
    long idx = 0;
    for (int k = 0; k < 4; k++) {
      int c = (t.n[k] <= 1) ? 0 : ind[k] + b[k];
      idx = idx * t.n[k] + c;
    }
    const double* node = &t.f[(size_t)idx * 17];
    for (int i = 0; i < 17; i++) out[i] += w * node[i];
    if (jac)
      for (int j = 0; j < 4; j++) {
        double dw = (1.0 - 2.0 * b[j]) * dfr[j];
        for (int k = 0; k < 4; k++)
          if (k != j) dw *= wk[k];
        for (int f = 0; f < 5; f++) jac[f][j] += dw * node[1 + f];
      }
  }
}

inline void table_box(const Table& t, double* lo, double* hi) {
  for (int k = 0; k < 4; k++) {
    lo[k] = t.lo[k];
    hi[k] = t.lo[k] + t.d[k] * (t.n[k] - 1);
  }
}

}  // namespace orc
