// EoS kernels of the GB300 SPH hot path: the per-particle inversion after the
// smoothing pass (FP64 form), the initial inversion of the input densities,
// and the batch inversion / thermodynamics entry points. Kept in their own
// translation unit: the inverter and its chain of models are the largest
// code in the library, and apart from the pass kernels they compile in
// parallel.
#include "kernels.cuh"
#include "passes.cuh"
#include "physics.cuh"

namespace ccake {

namespace {

using namespace passes;

template <int D, bool DIFF>
__global__ void __launch_bounds__(kBlock) k_thermo(RunConst rc, EosDev eos, Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  thermo_tail<D, false, DIFF>(rc, eos, p, i, p.clock->t);
}

// The same for an EoS of kind KIND known at launch (an analytic model, no
// pre-inverted tables): the kind in a local copy is a constant, so the
// chain's table and tanh-conformal code drops out of the kernel and the
// inversion of the same model runs in fewer registers.
template <int D, bool DIFF, int KIND>
__global__ void __launch_bounds__(kBlock) k_thermo_kind(RunConst rc, EosDev eos, Ptrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  EosDev e = eos;
  e.kind = KIND;
  e.pre = nullptr;
  thermo_tail<D, false, DIFF>(rc, e, p, i, p.clock->t);
}

// seeds (n rows of T, muB, muQ, muS, or null): the learned seed of every
// particle, tried first on the first model of the chain
__global__ void k_init_invert(RunConst rc, EosDev eos, Ptrs p, const double* seeds) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int n = p.n;
  const int entropy = rc.cfg.input_as_entropy;
  double x[4] = {p.th[T_T * n + i], 0.0, 0.0, 0.0};
  if (seeds)
    for (int q = 0; q < 4; q++) x[q] = seeds[(size_t)4 * i + q];
  double tgt[4] = {p.in_e[i], p.in_rho[i], p.in_rho[n + i], p.in_rho[2 * n + i]};
  int iters = 0;
  int k = eos_invert(eos, entropy, tgt, 0, x, &iters, seeds ? 2 : 0);
  if (k < 0 && !entropy) {
    // freeze the particle and retry at zero charge (src/sph_workstation.cpp:1825-1848)
    p.freeze[i] = 4;
    x[0] = p.th[T_T * n + i]; x[1] = x[2] = x[3] = 0.0;
    const double tz[4] = {tgt[0], 0.0, 0.0, 0.0};
    k = eos_invert(eos, 0, tz, 0, x, &iters);
  }
  if (k < 0) {   // per-particle status: no EoS solution
    p.eos_id[i] = -1;
    flag_error(p.err, E_EOS);
    return;
  }
  double th[NTH];
  set_thermo(eos, k, x, th);
  for (int q = 0; q < NTH; q++) p.th[q * n + i] = th[q];
  p.eos_id[i] = k;
  p.eos_iters[i] = iters;
  if (entropy) { p.in_s[i] = p.in_e[i]; p.in_e[i] = th[T_E]; }
  else p.in_s[i] = th[T_S];
  if (!(p.in_e[i] > rc.efreeze && p.freeze[i] != 4)) p.freeze[i] = 4;
}

__global__ void k_eos_thermo(EosDev eos, int model, int64_t n, const double* tbqs, double* out17) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  model_thermo(eos, model, tbqs + 4 * i, out17 + 17 * i);
}

// Pass 1 of the two-pass batch inversion: the first attempt of each row
// with a Newton budget; rows it does not settle are appended to `list` (an
// atomic append: rows are independent, so the order does not matter).
__global__ void k_eos_first(EosDev eos, int entropy, int seed_mode, int max_it, int64_t n, const double* in4,
                            double* tbqs, double* th16, int32_t* status, int32_t* iters, int32_t* list,
                            int32_t* count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[4] = {tbqs[4 * i], tbqs[4 * i + 1], tbqs[4 * i + 2], tbqs[4 * i + 3]};
  int it = 0;
  double o[17];
  const int k = eos_invert_first(eos, entropy, in4 + 4 * i, 0, x, &it, seed_mode, max_it, o);
  if (k == -2) {
    list[atomicAdd(count, 1)] = (int32_t)i;
    return;
  }
  status[i] = k;
  if (iters) iters[i] = it;
  for (int q = 0; q < 4; q++) tbqs[4 * i + q] = x[q];
  if (th16) set_thermo_o(eos, k, x, o, th16 + 16 * i);
}

// Pass 2: the full inversion of the listed rows.
__global__ void k_eos_rest(EosDev eos, int entropy, int seed_mode, const int32_t* list, const int32_t* count,
                           const double* in4, double* tbqs, double* th16, int32_t* status, int32_t* iters) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *count) return;
  const int64_t i = list[j];
  double x[4] = {tbqs[4 * i], tbqs[4 * i + 1], tbqs[4 * i + 2], tbqs[4 * i + 3]};
  int it = 0;
  double o[17];
  const int k = eos_invert(eos, entropy, in4 + 4 * i, 0, x, &it, seed_mode, o);
  status[i] = k;
  if (iters) iters[i] = it;
  if (k >= 0) {
    for (int q = 0; q < 4; q++) tbqs[4 * i + q] = x[q];
    if (th16) set_thermo_o(eos, k, x, o, th16 + 16 * i);
  }
}

__global__ void k_eos_batch(EosDev eos, int entropy, int seed_mode, int64_t n, const double* in4, double* tbqs,
                            double* th16, int32_t* status, int32_t* iters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[4] = {tbqs[4 * i], tbqs[4 * i + 1], tbqs[4 * i + 2], tbqs[4 * i + 3]};
  int it = 0;
  double o[17];
  const int k = eos_invert(eos, entropy, in4 + 4 * i, 0, x, &it, seed_mode, o);
  status[i] = k;
  if (iters) iters[i] = it;
  if (k >= 0) {
    for (int q = 0; q < 4; q++) tbqs[4 * i + q] = x[q];
    if (th16) set_thermo_o(eos, k, x, o, th16 + 16 * i);
  }
}

}  // namespace

void launch_thermo(const RunConst& rc, const EosDev& eos, const Ptrs& p, cudaStream_t s) {
  const int nb = (p.n + kBlock - 1) / kBlock;
  const bool dif = rc.cfg.using_diffusion && p.dif;
  if (rc.cfg.dim == 3) {
    if (dif) k_thermo<3, true><<<nb, kBlock, 0, s>>>(rc, eos, p);
    else k_thermo<3, false><<<nb, kBlock, 0, s>>>(rc, eos, p);
  } else if (eos.kind == 1 && !eos.pre) {
    if (dif) k_thermo_kind<2, true, 1><<<nb, kBlock, 0, s>>>(rc, eos, p);
    else k_thermo_kind<2, false, 1><<<nb, kBlock, 0, s>>>(rc, eos, p);
  } else {
    if (dif) k_thermo<2, true><<<nb, kBlock, 0, s>>>(rc, eos, p);
    else k_thermo<2, false><<<nb, kBlock, 0, s>>>(rc, eos, p);
  }
}

void launch_init_invert(const RunConst& rc, const EosDev& eos, const Ptrs& p, const double* seeds, cudaStream_t s) {
  k_init_invert<<<(p.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(rc, eos, p, seeds);
}

void launch_eos_thermo(const EosDev& eos, int chain_index, int64_t n, const double* tbqs, double* out17,
                       cudaStream_t s) {
  const int nb = (int)((n + kBlock - 1) / kBlock);
  k_eos_thermo<<<nb, kBlock, 0, s>>>(eos, chain_model(eos.kind, chain_index), n, tbqs, out17);
}

void launch_eos_batch(const EosDev& eos, int entropy, int seed_mode, int64_t n, const double* in4, double* tbqs,
                      double* th16, int32_t* status, int32_t* iters, int32_t* scratch, cudaStream_t s) {
  const int nb = (int)((n + kBlock - 1) / kBlock);
  if (seed_mode == 1 || !scratch) {
    k_eos_batch<<<nb, kBlock, 0, s>>>(eos, entropy, seed_mode, n, in4, tbqs, th16, status, iters);
    return;
  }
  // two passes: a warp of the single-pass kernel runs as long as its slowest
  // row; the capped first pass settles most rows in a few Newton steps and
  // the compacted second pass gives the hard rows warps of their own
  int32_t* count = scratch;
  int32_t* list = scratch + 1;
  cudaMemsetAsync(count, 0, sizeof(int32_t), s);
  k_eos_first<<<nb, kBlock, 0, s>>>(eos, entropy, seed_mode, kEosFirstIters, n, in4, tbqs, th16, status, iters, list,
                                    count);
  k_eos_rest<<<nb, kBlock, 0, s>>>(eos, entropy, seed_mode, list, count, in4, tbqs, th16, status, iters);
}

}  // namespace ccake
