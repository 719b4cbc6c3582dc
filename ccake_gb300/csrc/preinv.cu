// Pre-inverted (s, rhoB, rhoS, rhoQ) -> thermodynamics tables on the device:
// the reference's table generator (utilities/generate_eos_table.cpp:228-342)
// and its lookup (src/eos_interpolator.cpp:531-739, preinv_lookup in
// eos.cuh). The generator inverts every node of a chunk of tiles at once with
// the batched entropy-mode inversion, from the generator's seed
// (T = 750/197 fm^-1, mu = 0), and packs the 11 tabulated values.
#include "kernels.cuh"
#include "passes.cuh"

namespace ccake {

namespace {



// densities of the nodes of tiles [tile0, tile0 + ntiles): x = min + i * step
// (generate_eos_table.cpp:305-308, roundings explicit)
__global__ void k_preinv_grid(PreinvView P, int64_t tile0, int64_t count, double* in4, double* tbqs) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= count) return;
  const int64_t N = P.N, tn = N * N * N * N;
  const int64_t tile = tile0 + g / tn, node = g % tn;
  int t[4], ix[4];
  int64_t r = tile;
  for (int k = 3; k >= 0; k--) { t[k] = (int)(r % P.nt[k]); r /= P.nt[k]; }
  r = node;
  for (int k = 3; k >= 0; k--) { ix[k] = (int)(r % N); r /= N; }
  for (int k = 0; k < 4; k++) in4[4 * g + k] = __dadd_rn(P.mn[k][t[k]], __dmul_rn((double)ix[k], P.st[k][t[k]]));
  tbqs[4 * g] = 750. / 197.;
  tbqs[4 * g + 1] = tbqs[4 * g + 2] = tbqs[4 * g + 3] = 0.0;
}

// th16 (T muB muS muQ p s rhoB rhoS rhoQ e w cs2 dwds dwdB dwdS dwdQ) -> the
// 11 tabulated values; a node without a solution is NaN and counted
__global__ void k_preinv_pack(int64_t count, const double* th16, const int32_t* status, double* out, int32_t* nfail) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= count) return;
  double* o = out + (size_t)g * kPreVars;
  if (status[g] < 0) {
    for (int v = 0; v < kPreVars; v++) o[v] = NAN;
    atomicAdd(nfail, 1);
    return;
  }
  const double* th = th16 + 16 * g;
  o[PV_T] = th[T_T];
  o[PV_MUB] = th[T_MUB];
  o[PV_MUQ] = th[T_MUQ];
  o[PV_MUS] = th[T_MUS];
  o[PV_E] = th[T_E];
  o[PV_P] = th[T_P];
  o[PV_CS2] = th[T_CS2];
  o[PV_DWDS] = th[T_DWDS];
  o[PV_DWDB] = th[T_DWDB];
  o[PV_DWDQ] = th[T_DWDQ];
  o[PV_DWDS_S] = th[T_DWDSS];
}

__global__ void k_preinv_lookup(const PreinvView* P, int64_t n, const double* sBSQ, double* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[kPreVars];
  preinv_lookup(*P, sBSQ + 4 * i, v);
  for (int q = 0; q < kPreVars; q++) out[(size_t)i * kPreVars + q] = v[q];
}

}  // namespace

void launch_preinv_grid(const PreinvView& P, int64_t tile0, int64_t count, double* in4, double* tbqs,
                        cudaStream_t s) {
  if (count <= 0) return;
  k_preinv_grid<<<(unsigned)((count + kBlock - 1) / kBlock), kBlock, 0, s>>>(P, tile0, count, in4, tbqs);
}

void launch_preinv_pack(int64_t count, const double* th16, const int32_t* status, double* out, int32_t* nfail,
                        cudaStream_t s) {
  if (count <= 0) return;
  k_preinv_pack<<<(unsigned)((count + kBlock - 1) / kBlock), kBlock, 0, s>>>(count, th16, status, out, nfail);
}

void launch_preinv_lookup(const PreinvView* P, int64_t n, const double* sBSQ, double* out, cudaStream_t s) {
  if (n <= 0) return;
  k_preinv_lookup<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(P, n, sBSQ, out);
}

}  // namespace ccake
