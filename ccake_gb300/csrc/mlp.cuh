// Learned Newton seed for the tabulated EoS: a 4-64-64-64-4 tanh MLP mapping
// (log e, rho_i / e^(3/4)) to (log T, mu_i / T), both standardised, trained
// and evaluated with BF16 tensor-core (tcgen05) kernels.
#pragma once
#include <cstdint>

#include "eos.cuh"

namespace ccake {

// FP32 parameter block (offsets in floats): W1 [64][4], b1 [64], W2 [64][64],
// b2 [64], W3 [64][64], b3 [64], W4 [4][64], b4 [4]; W[n][k] = weight from
// input k to output n.
namespace mlp {
constexpr int kW1 = 0, kB1 = 256, kW2 = 320, kB2 = 4416, kW3 = 4480, kB3 = 8576, kW4 = 8640, kB4 = 8896;
constexpr int kParams = 8900;
constexpr int kTile = 128;   // rows per tile (the MMA M and the CTA's thread count)
}  // namespace mlp

// Standardisation: feature f -> (f - in_mean) / in_std; network output o ->
// o * out_std + out_mean.
struct MlpNorm {
  float in_mean[4], in_std[4], out_mean[4], out_std[4];
};

struct MlpDev {
  const float* params = nullptr;   // kParams FP32 (device)
  MlpNorm norm{};
};

// Raw forward of n feature rows (standardised inputs in, standardised
// outputs out; device arrays of n x 4 floats).
void launch_mlp_forward(const float* params, int64_t n, const float* feat, float* out, int32_t* err, cudaStream_t s);

// One gradient evaluation: d(mean squared error)/d(params) over n rows,
// accumulated into grads (kParams floats, zeroed by the caller) and the sum
// of squared errors into sse (double, zeroed by the caller).
void launch_mlp_grad(const float* params, int64_t n, const float* feat, const float* tgt, float* grads, double* sse,
                     int32_t* err, cudaStream_t s);

// Adam step on the FP32 parameters (bias-corrected, step t >= 1).
void launch_mlp_adam(float* params, const float* grads, float* m, float* v, float lr, int t, cudaStream_t s);

// Training samples: states uniform in the table box (counter-based hash RNG
// from seed), mapped forward through the table; features and targets before
// standardisation, invalid rows (non-finite fields, e <= 0) flagged 0 in ok.
void launch_mlp_samples(const EosDev& eos, int64_t n, uint64_t seed, float* feat, float* tgt, int32_t* ok,
                        cudaStream_t s);

// Standardises n rows in place: feat with in_*, tgt with out_*.
void launch_mlp_standardise(const MlpNorm& nm, int64_t n, float* feat, float* tgt, cudaStream_t s);

// Seeds (T, muB, muQ, muS) for n energy-mode rows (e, rhoB, rhoS, rhoQ) from
// the network; rows with e <= 0 keep their seed.
void launch_mlp_seed(const MlpDev& m, int64_t n, const double* in4, double* tbqs, int32_t* err, cudaStream_t s);

int mlp_smem_forward();
int mlp_smem_grad();

}  // namespace ccake
