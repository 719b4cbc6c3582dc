// Neighbour counts without any device allocation.
//
// For callers that cannot allocate device memory while they run: code that
// calls in from inside another library's allocation-free region, from a host
// callback or a stream-ordered section where cudaMalloc would synchronise or
// is forbidden, or from a process whose allocator is owned by someone else.
// They pass device positions and a device output array; the cell-list scratch
// lives in the file-scope array below, sized for at most kMaxParticles
// particles and kMaxCells cells (about 5.2 MB, held by every device that loads
// the library until the process exits).
//
// Contract:
//  * The first call on each device looks up the device address of the scratch
//    array with cudaGetSymbolAddress (with that device current) and caches it;
//    make that first call before any stream capture. The cache assumes that
//    the device's primary context lives as long as the process: after a
//    cudaDeviceReset the module is loaded again and the cached address is
//    stale, so a caller that resets a device must not call this entry point
//    on it afterwards.
//  * All calls share the one scratch array and it keeps the last call's
//    contents; every call clears the cell counters it uses before binning.
//    Calls that overlap on the GPU (different streams, or different host
//    threads) race on the scratch and give wrong counts: serialise them.
//  * Sizes beyond kMaxParticles / kMaxCells are rejected with
//    CCAKE_ERR_CAPACITY before anything is launched.
#include <cmath>
#include <mutex>

#include "ccake_gpu.h"
#include "common.cuh"

namespace ccake {
namespace {

constexpr int64_t kMaxParticles = 1 << 18;
constexpr int64_t kMaxCells = 1 << 18;
// cell_of | rank | sorted index (kMaxParticles each) | count | start (kMaxCells + 1)
constexpr int64_t kScratchInts = 3 * kMaxParticles + 2 * kMaxCells + 1;

static __device__ __align__(256) int32_t g_noalloc_scratch[kScratchInts];

constexpr int kMaxDevices = 64;
int32_t* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

struct Scratch {
  int32_t *cell_of, *rank, *idx, *count, *start;
};

Scratch carve(int32_t* base) {
  Scratch s;
  s.cell_of = base;
  s.rank = base + kMaxParticles;
  s.idx = base + 2 * kMaxParticles;
  s.count = base + 3 * kMaxParticles;
  s.start = base + 3 * kMaxParticles + kMaxCells;
  return s;
}

__global__ void na_zero(int32_t* a, int m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) a[i] = 0;
}

__device__ __forceinline__ int na_cell(const Grid& g, const double* x, const double* y, const double* z, int dim, int i) {
  int c = cell_coord(g, 0, x[i]) + g.nc[0] * cell_coord(g, 1, y[i]);
  if (dim == 3) c += g.nc[0] * g.nc[1] * cell_coord(g, 2, z[i]);
  return c;
}

__global__ void na_bin(Grid g, const double* x, const double* y, const double* z, int dim, int n, Scratch s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = na_cell(g, x, y, z, dim, i);
  s.cell_of[i] = c;
  s.rank[i] = atomicAdd(&s.count[c], 1);
}

__global__ void na_scan(Scratch s, int ncell) {
  __shared__ int32_t part[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int chunk = (ncell + nt - 1) / nt;
  const int b = tid * chunk, e = min(ncell, b + chunk);
  int32_t local = 0;
  for (int c = b; c < e; c++) local += s.count[c];
  part[tid] = local;
  __syncthreads();
  if (tid == 0) {
    int32_t run = 0;
    for (int k = 0; k < nt; k++) { const int32_t v = part[k]; part[k] = run; run += v; }
    s.start[ncell] = run;
  }
  __syncthreads();
  int32_t run = part[tid];
  for (int c = b; c < e; c++) { s.start[c] = run; run += s.count[c]; }
}

__global__ void na_scatter(Scratch s, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  s.idx[s.start[s.cell_of[i]] + s.rank[i]] = i;
}

__global__ void na_count(Grid g, const double* x, const double* y, const double* z, int dim, int n, double cut2,
                         Scratch s, int32_t* counts) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const double xa[3] = {x[a], y[a], dim == 3 ? z[a] : 0.0};
  const int cx = cell_coord(g, 0, xa[0]), cy = cell_coord(g, 1, xa[1]);
  const int cz = dim == 3 ? cell_coord(g, 2, xa[2]) : 0;
  int cnt = 0;
  for (int k = max(cz - 1, 0); k <= min(cz + 1, g.nc[2] - 1); k++)
    for (int j = max(cy - 1, 0); j <= min(cy + 1, g.nc[1] - 1); j++) {
      const int row = (k * g.nc[1] + j) * g.nc[0];
      const int jb = s.start[row + max(cx - 1, 0)], je = s.start[row + min(cx + 1, g.nc[0] - 1) + 1];
      for (int q = jb; q < je; q++) {
        const int b = s.idx[q];
        if (b == a) continue;
        double d[3] = {xa[0] - x[b], xa[1] - y[b], dim == 3 ? xa[2] - z[b] : 0.0};
        const double d2 = dim == 3 ? dist2_exact<3>(d) : dist2_exact<2>(d);
        if (d2 <= cut2) cnt++;
      }
    }
  counts[a] = cnt;
}

// Device address of the scratch array for the current device (cached).
ccake_status_t scratch_for_current_device(int32_t** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CCAKE_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return CCAKE_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<int32_t*>(ptr);
  }
  *out = g_scratch_addr[dev];
  return CCAKE_OK;
}

}  // namespace
}  // namespace ccake

using namespace ccake;

extern "C" ccake_status_t ccake_neighbour_counts_noalloc(const double* d_x, const double* d_y, const double* d_eta,
                                                         int64_t n, int32_t dim, double h, const double* lo3,
                                                         const double* hi3, int32_t* d_counts, void* stream) {
  if (!d_x || !d_y || !d_counts || !lo3 || !hi3 || n <= 0 || !(h > 0)) return CCAKE_ERR_INVALID;
  if (dim != 2 && dim != 3) return CCAKE_ERR_INVALID;
  if (dim == 3 && !d_eta) return CCAKE_ERR_INVALID;
  if (n > kMaxParticles) return CCAKE_ERR_CAPACITY;
  // cell grid over the caller's box, indices clamped. The cell edge is kept
  // strictly above 2h (by a relative margin of 1e-9): with an edge of exactly
  // 2h, floor((x - lo) * inv_cs) of two particles exactly 2h apart -- four
  // such pairs around every lattice particle -- can round into cells two
  // apart, and the pair would be missed.
  Grid g{};
  const double cut = 2.0 * h;
  int64_t ncell = 1;
  for (int k = 0; k < 3; k++) {
    if (k >= dim) { g.lo[k] = 0.0; g.nc[k] = 1; g.inv_cs[k] = 1.0; continue; }
    if (!(hi3[k] > lo3[k])) return CCAKE_ERR_INVALID;
    const double span = hi3[k] - lo3[k];
    const double ncd = std::floor(span / (cut * (1.0 + 1e-9)));
    if (!(ncd <= (double)kMaxCells)) return CCAKE_ERR_CAPACITY;
    const int nc = ncd < 1.0 ? 1 : (int)ncd;
    g.lo[k] = lo3[k];
    g.nc[k] = nc;
    g.inv_cs[k] = nc / span;
    ncell *= nc;
  }
  if (ncell > kMaxCells) return CCAKE_ERR_CAPACITY;
  g.ncell = (int)ncell;
  int32_t* base = nullptr;
  ccake_status_t st = scratch_for_current_device(&base);
  if (st != CCAKE_OK) return st;
  Scratch s = carve(base);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const int nn = (int)n, nb = (nn + 127) / 128;
  na_zero<<<(g.ncell + 255) / 256, 256, 0, cs>>>(s.count, g.ncell);
  na_bin<<<nb, 128, 0, cs>>>(g, d_x, d_y, d_eta, dim, nn, s);
  na_scan<<<1, 1024, 0, cs>>>(s, g.ncell);
  na_scatter<<<nb, 128, 0, cs>>>(s, nn);
  na_count<<<nb, 128, 0, cs>>>(g, d_x, d_y, d_eta, dim, nn, cut * cut, s, d_counts);
  return cudaGetLastError() == cudaSuccess ? CCAKE_OK : CCAKE_ERR_CUDA;
}
