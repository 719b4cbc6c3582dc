// Learned Newton seed for the tabulated EoS: BF16 tensor-core (tcgen05)
// kernels for the forward pass, the gradient of the squared error and the
// seeds of a batch inversion, plus the Adam step and the sample generator.
//
// One CTA of 128 threads per 128-row tile; thread t owns row t and TMEM lane
// t. Every layer is one tcgen05.mma group (M = 128, K = 16 per instruction)
// issued by thread 0 on BF16 operands in shared memory (K-major, no swizzle:
// 8 x 16-byte core matrices, SBO = 128 B between 8-row groups, LBO between
// 16-byte K chunks) with an FP32 accumulator in TMEM, completed through an
// mbarrier and read back with tcgen05.ld. Weight gradients of the two
// 64 x 64 layers are tensor-core GEMMs over the batch (transposed
// activations as operands, accumulated in TMEM across a CTA's tiles); the
// 4-wide first and last layers and the biases reduce on the CUDA cores.
// Every mbarrier wait has an iteration limit; on expiry the kernel records
// the error, frees its TMEM and returns.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>

#include "kernels.cuh"
#include "mlp.cuh"

namespace ccake {

namespace {

using namespace mlp;

// ---------------------------------------------------------------------------
// tcgen05 / mbarrier primitives (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between K chunks), stride byte offset 128 (between 8-row groups),
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)(128u >> 4) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the mbarrier phase `parity` to complete.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (uint32_t i = 0; i < (1u << 24); i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// operand layouts
// ---------------------------------------------------------------------------
// Byte offset of element (r, k) of a K-major operand with R rows (R % 8 == 0).
__host__ __device__ constexpr uint32_t koff(int r, int k, int R) {
  return (uint32_t)((k >> 3) * (R >> 3) * 128 + (r >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v) {
  *reinterpret_cast<unsigned short*>(base + off) = __bfloat16_as_ushort(__float2bfloat16_rn(v));
}
__device__ __forceinline__ float ld_bf16(const unsigned char* base, uint32_t off) {
  return __bfloat162float(__ushort_as_bfloat16(*reinterpret_cast<const unsigned short*>(base + off)));
}
__device__ __forceinline__ float bf16_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// Row r of a K-major operand with R rows: 8 k-values starting at k0 (k0 % 8
// == 0) in one 16-byte store.
__device__ __forceinline__ void st_row8(unsigned char* base, int r, int k0, int R, const float* v) {
  uint4 q;
  q.x = pack2(v[0], v[1]);
  q.y = pack2(v[2], v[3]);
  q.z = pack2(v[4], v[5]);
  q.w = pack2(v[6], v[7]);
  *reinterpret_cast<uint4*>(base + koff(r, k0, R)) = q;
}

// D (TMEM column dcol) [128 x N] (+)= A [128 x K] * B [N x K]^T; A has RA
// rows in its layout (>= 128 lanes used), B has N rows.
__device__ __forceinline__ void gemm(uint32_t tmem, int dcol, uint32_t a, int RA, uint32_t b, int N, int K,
                                     bool accumulate) {
  const uint32_t lboA = (uint32_t)(RA >> 3) * 128u, lboB = (uint32_t)(N >> 3) * 128u;
  const uint32_t id = idesc_bf16(128, N);
  for (int s = 0; s < K / 16; s++)
    umma(tmem + (uint32_t)dcol, sdesc(a + 2u * s * lboA, lboA), sdesc(b + 2u * s * lboB, lboB), id,
         (accumulate || s > 0) ? 1u : 0u);
}

// Reduce-scatter of N values per lane over the warp (N % 32 == 0): after it
// the lane holds in v[0 .. N/32) the warp sums of indices rs_base(lane, N) + j.
template <int N>
__device__ __forceinline__ void warp_reduce_scatter(float (&v)[N], int lane) {
#pragma unroll
  for (int r = 0; r < 5; r++) {
    const int o = 16 >> r;
    const int half = N >> (r + 1);
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < half; i++) {
      const float send = up ? v[i] : v[i + half];
      const float keep = up ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
}
__device__ __forceinline__ int rs_base(int lane, int N) {
  int b = 0;
#pragma unroll
  for (int r = 0; r < 5; r++)
    if (lane & (16 >> r)) b += N >> (r + 1);
  return b;
}

// ---------------------------------------------------------------------------
// shared-memory plans (byte offsets)
// ---------------------------------------------------------------------------
struct FwdPlan {
  static constexpr uint32_t W1 = 0;                 // 64 x 16
  static constexpr uint32_t W2 = W1 + 64 * 16 * 2;  // 64 x 64
  static constexpr uint32_t W3 = W2 + 64 * 64 * 2;
  static constexpr uint32_t W4 = W3 + 64 * 64 * 2;  // 16 x 64
  static constexpr uint32_t A0 = W4 + 16 * 64 * 2;  // 128 x 16
  static constexpr uint32_t P = A0 + 128 * 16 * 2;  // 128 x 64
  static constexpr uint32_t Q = P + 128 * 64 * 2;
  static constexpr uint32_t BIAS = Q + 128 * 64 * 2;  // b1 b2 b3 (64 each) b4 (16), FP32
  static constexpr uint32_t MISC = BIAS + 208 * 4;    // mbarrier (8), TMEM address (4)
  static constexpr uint32_t BYTES = MISC + 64;
};

struct GradPlan {
  static constexpr uint32_t W1 = 0;
  static constexpr uint32_t W2 = W1 + 64 * 16 * 2;
  static constexpr uint32_t W3 = W2 + 64 * 64 * 2;
  static constexpr uint32_t W4 = W3 + 64 * 64 * 2;   // 16 x 64
  static constexpr uint32_t W2T = W4 + 16 * 64 * 2;  // 64 x 64, element (k, n) = W2[n][k]
  static constexpr uint32_t W3T = W2T + 64 * 64 * 2;
  static constexpr uint32_t W4T = W3T + 64 * 64 * 2;  // 64 x 16, element (k, n) = W4[n][k]
  static constexpr uint32_t A0 = W4T + 64 * 16 * 2;   // 128 x 16
  static constexpr uint32_t P = A0 + 128 * 16 * 2;    // 128 x 64
  static constexpr uint32_t Q = P + 128 * 64 * 2;
  static constexpr uint32_t HT1 = Q + 128 * 64 * 2;   // 64 features x 128 rows
  static constexpr uint32_t HT2 = HT1 + 64 * 128 * 2;
  static constexpr uint32_t HT3 = HT2 + 64 * 128 * 2;
  static constexpr uint32_t DO = HT3 + 64 * 128 * 2;  // 128 x 16
  static constexpr uint32_t DZT = DO + 128 * 16 * 2;  // 128 (64 features + 64 zero) x 128 rows
  static constexpr uint32_t BIAS = DZT + 128 * 128 * 2;
  static constexpr uint32_t ACC = BIAS + 208 * 4;     // dW1 [256] dW4 [256] db1 db2 db3 [64 each] db4 [4]
  static constexpr uint32_t MISC = ACC + 708 * 4;
  static constexpr uint32_t BYTES = MISC + 64;
};

// Weights from the FP32 parameters into BF16 B operands (rows = outputs).
template <class Plan>
__device__ void load_weights(const float* __restrict__ prm, unsigned char* sm, bool transposed) {
  const int t = threadIdx.x;
  for (int i = t; i < 64 * 16; i += blockDim.x) {   // W1 [64][16], k >= 4 zero
    const int nn = i / 16, k = i % 16;
    st_bf16(sm, Plan::W1 + koff(nn, k, 64), k < 4 ? prm[kW1 + nn * 4 + k] : 0.0f);
  }
  for (int i = t; i < 64 * 64; i += blockDim.x) {
    const int nn = i / 64, k = i % 64;
    st_bf16(sm, Plan::W2 + koff(nn, k, 64), prm[kW2 + i]);
    st_bf16(sm, Plan::W3 + koff(nn, k, 64), prm[kW3 + i]);
  }
  for (int i = t; i < 16 * 64; i += blockDim.x) {   // W4 [16][64], n >= 4 zero
    const int nn = i / 64, k = i % 64;
    st_bf16(sm, Plan::W4 + koff(nn, k, 16), nn < 4 ? prm[kW4 + nn * 64 + k] : 0.0f);
  }
  float* bias = reinterpret_cast<float*>(sm + Plan::BIAS);
  for (int i = t; i < 208; i += blockDim.x)
    bias[i] = i < 64 ? prm[kB1 + i] : (i < 128 ? prm[kB2 + i - 64] : (i < 192 ? prm[kB3 + i - 128] : (i < 196 ? prm[kB4 + i - 192] : 0.0f)));
  (void)transposed;
}

__device__ void load_transposed(const float* __restrict__ prm, unsigned char* sm) {
  const int t = threadIdx.x;
  for (int i = t; i < 64 * 64; i += blockDim.x) {   // element (k, n) = W[n][k]
    const int nn = i / 64, k = i % 64;
    st_bf16(sm, GradPlan::W2T + koff(k, nn, 64), prm[kW2 + i]);
    st_bf16(sm, GradPlan::W3T + koff(k, nn, 64), prm[kW3 + i]);
  }
  for (int i = t; i < 64 * 16; i += blockDim.x) {   // W4T [64][16], n >= 4 zero
    const int k = i / 16, nn = i % 16;
    st_bf16(sm, GradPlan::W4T + koff(k, nn, 64), nn < 4 ? prm[kW4 + nn * 64 + k] : 0.0f);
  }
}

// Issues the MMAs of one step (by thread 0, after a CTA barrier that makes
// the operand stores visible to the tensor core) and waits for them.
template <class Issue>
__device__ __forceinline__ bool mma_step(uint32_t mbar, uint32_t& phase, Issue&& issue) {
  proxy_fence();
  tc_before_sync();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_after_sync();
    issue();
    umma_commit(mbar);
  }
  bool ok = mbar_wait(mbar, phase);
  phase ^= 1u;
  ok = __syncthreads_and(ok) != 0;
  tc_after_sync();
  return ok;
}

// tanh layer epilogue: this thread's 64 accumulator columns + bias -> tanh.
__device__ __forceinline__ void act_row(uint32_t tlane, const float* bias, float* h) {
#pragma unroll
  for (int c = 0; c < 4; c++) tmem_ld16(tlane + 16 * c, h + 16 * c);
#pragma unroll
  for (int k = 0; k < 64; k++) h[k] = tanhf(h[k] + bias[k]);
}

// ---------------------------------------------------------------------------
// forward / seed kernel
// ---------------------------------------------------------------------------
template <bool SEED>
__global__ void __launch_bounds__(128) k_mlp_fwd(const float* __restrict__ prm, MlpNorm nm, int64_t n,
                                                 const float* __restrict__ feat, float* __restrict__ out,
                                                 const double* __restrict__ in4, double* __restrict__ tbqs,
                                                 int32_t* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  using PL = FwdPlan;
  const int t = threadIdx.x, warp = t >> 5;
  load_weights<PL>(prm, sm, false);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + PL::MISC + 8);
  const uint32_t mbar = smem_u32(sm + PL::MISC);
  if (t == 0) mbar_init(mbar);
  if (warp == 0) tmem_alloc(smem_u32(tslot), 64);
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
  const float* bias = reinterpret_cast<const float*>(sm + PL::BIAS);
  const uint32_t sA0 = smem_u32(sm + PL::A0), sP = smem_u32(sm + PL::P), sQ = smem_u32(sm + PL::Q);
  const uint32_t sW1 = smem_u32(sm + PL::W1), sW2 = smem_u32(sm + PL::W2), sW3 = smem_u32(sm + PL::W3),
                 sW4 = smem_u32(sm + PL::W4);
  uint32_t phase = 0;
  const int64_t ntiles = (n + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t row = tile * kTile + t;
    const bool valid = row < n;
    float x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = 0.0f;
    bool use = valid;
    if (valid) {
      if (SEED) {
        const double e = in4[4 * row];
        use = e > 0.0 && isfinite(e);
        const double ie34 = use ? pow(e, -0.75) : 0.0;
        const double f[4] = {use ? log(e) : 0.0, in4[4 * row + 1] * ie34, in4[4 * row + 2] * ie34,
                             in4[4 * row + 3] * ie34};
#pragma unroll
        for (int k = 0; k < 4; k++) x[k] = use ? ((float)f[k] - nm.in_mean[k]) / nm.in_std[k] : 0.0f;
      } else {
#pragma unroll
        for (int k = 0; k < 4; k++) x[k] = feat[4 * row + k];
      }
    }
    st_row8(sm + PL::A0, t, 0, 128, x);
    st_row8(sm + PL::A0, t, 8, 128, x + 8);
    float h[64];
    bool ok = mma_step(mbar, phase, [&] { gemm(tmem, 0, sA0, 128, sW1, 64, 16, false); });
    if (ok) {
      act_row(tlane, bias, h);
#pragma unroll
      for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::P, t, k0, 128, h + k0);
      ok = mma_step(mbar, phase, [&] { gemm(tmem, 0, sP, 128, sW2, 64, 64, false); });
    }
    if (ok) {
      act_row(tlane, bias + 64, h);
#pragma unroll
      for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::Q, t, k0, 128, h + k0);
      ok = mma_step(mbar, phase, [&] { gemm(tmem, 0, sQ, 128, sW3, 64, 64, false); });
    }
    if (ok) {
      act_row(tlane, bias + 128, h);
#pragma unroll
      for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::P, t, k0, 128, h + k0);
      ok = mma_step(mbar, phase, [&] { gemm(tmem, 0, sP, 128, sW4, 16, 64, false); });
    }
    if (!ok) {
      if (t == 0) atomicExch(err, 1);
      break;
    }
    float o[16];
    tmem_ld16(tlane, o);
    if (valid) {
      float y[4];
#pragma unroll
      for (int k = 0; k < 4; k++) y[k] = o[k] + bias[192 + k];
      if (SEED) {
        if (use) {
          const double lT = (double)y[0] * nm.out_std[0] + nm.out_mean[0];
          const double T = exp(lT);
          double s[4] = {T, 0, 0, 0};
#pragma unroll
          for (int k = 1; k < 4; k++) s[k] = ((double)y[k] * nm.out_std[k] + nm.out_mean[k]) * T;
          if (isfinite(T) && T > 0.0)
            for (int k = 0; k < 4; k++) tbqs[4 * row + k] = s[k];
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; k++) out[4 * row + k] = y[k];
      }
    }
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (warp == 0) tmem_dealloc(tmem, 64);
}

// ---------------------------------------------------------------------------
// gradient kernel
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_mlp_grad(const float* __restrict__ prm, int64_t n,
                                                  const float* __restrict__ feat, const float* __restrict__ tgt,
                                                  float* __restrict__ grads, double* sse_out, int32_t* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  using PL = GradPlan;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  load_weights<PL>(prm, sm, true);
  load_transposed(prm, sm);
  {
    uint4 z = make_uint4(0, 0, 0, 0);
    for (int i = t; i < 128 * 128 * 2 / 16; i += blockDim.x) reinterpret_cast<uint4*>(sm + PL::DZT)[i] = z;
    float* acc = reinterpret_cast<float*>(sm + PL::ACC);
    for (int i = t; i < 708; i += blockDim.x) acc[i] = 0.0f;
  }
  float* dW1s = reinterpret_cast<float*>(sm + PL::ACC);
  float* dW4s = dW1s + 256;
  float* db1s = dW4s + 256;
  float* db2s = db1s + 64;
  float* db3s = db2s + 64;
  float* db4s = db3s + 64;
  double* sse_s = reinterpret_cast<double*>(sm + PL::MISC + 16);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + PL::MISC + 8);
  const uint32_t mbar = smem_u32(sm + PL::MISC);
  if (t == 0) {
    mbar_init(mbar);
    *sse_s = 0.0;
  }
  if (warp == 0) tmem_alloc(smem_u32(tslot), 256);
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
  constexpr int D0 = 0, DW2 = 64, DW3 = 128;
  const float* bias = reinterpret_cast<const float*>(sm + PL::BIAS);
  const uint32_t sA0 = smem_u32(sm + PL::A0), sP = smem_u32(sm + PL::P), sQ = smem_u32(sm + PL::Q);
  const uint32_t sW1 = smem_u32(sm + PL::W1), sW2 = smem_u32(sm + PL::W2), sW3 = smem_u32(sm + PL::W3),
                 sW4 = smem_u32(sm + PL::W4), sW2T = smem_u32(sm + PL::W2T), sW3T = smem_u32(sm + PL::W3T),
                 sW4T = smem_u32(sm + PL::W4T);
  const uint32_t sHT1 = smem_u32(sm + PL::HT1), sHT2 = smem_u32(sm + PL::HT2), sDO = smem_u32(sm + PL::DO),
                 sDZT = smem_u32(sm + PL::DZT);
  const float inv = 1.0f / (4.0f * (float)n);
  uint32_t phase = 0;
  bool first = true, ok = true;
  double sse = 0.0;
  const int64_t ntiles = (n + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t row = tile * kTile + t;
    float x[16], y[4];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = 0.0f;
    bool valid = row < n;
    if (valid) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        x[k] = feat[4 * row + k];
        y[k] = tgt[4 * row + k];
        valid = valid && isfinite(x[k]) && isfinite(y[k]);
      }
    }
    if (!valid) {
#pragma unroll
      for (int k = 0; k < 4; k++) { x[k] = 0.0f; y[k] = 0.0f; }
    }
    st_row8(sm + PL::A0, t, 0, 128, x);
    st_row8(sm + PL::A0, t, 8, 128, x + 8);
    float xb[4];   // inputs as the tensor core sees them
#pragma unroll
    for (int k = 0; k < 4; k++) xb[k] = bf16_round(x[k]);
    float h[64];
    // ---- forward
    ok = mma_step(mbar, phase, [&] { gemm(tmem, D0, sA0, 128, sW1, 64, 16, false); });
    if (!ok) break;
    act_row(tlane + D0, bias, h);
#pragma unroll
    for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::P, t, k0, 128, h + k0);
#pragma unroll
    for (int k = 0; k < 64; k++) st_bf16(sm, PL::HT1 + koff(k, t, 64), h[k]);
    ok = mma_step(mbar, phase, [&] { gemm(tmem, D0, sP, 128, sW2, 64, 64, false); });
    if (!ok) break;
    act_row(tlane + D0, bias + 64, h);
#pragma unroll
    for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::Q, t, k0, 128, h + k0);
#pragma unroll
    for (int k = 0; k < 64; k++) st_bf16(sm, PL::HT2 + koff(k, t, 64), h[k]);
    ok = mma_step(mbar, phase, [&] { gemm(tmem, D0, sQ, 128, sW3, 64, 64, false); });
    if (!ok) break;
    act_row(tlane + D0, bias + 128, h);
#pragma unroll
    for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::P, t, k0, 128, h + k0);
#pragma unroll
    for (int k = 0; k < 64; k++) st_bf16(sm, PL::HT3 + koff(k, t, 64), h[k]);
    ok = mma_step(mbar, phase, [&] { gemm(tmem, D0, sP, 128, sW4, 16, 64, false); });
    if (!ok) break;
    // ---- output, loss, dL/do
    float o[16], dO[16];
    tmem_ld16(tlane + D0, o);
#pragma unroll
    for (int k = 0; k < 16; k++) dO[k] = 0.0f;
    float ssq = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float e = valid ? (o[k] + bias[192 + k] - y[k]) : 0.0f;
      ssq += e * e;
      dO[k] = 2.0f * e * inv;
    }
    sse += (double)ssq;
    st_row8(sm + PL::DO, t, 0, 128, dO);
    st_row8(sm + PL::DO, t, 8, 128, dO + 8);
    // bf16 H3 of this row (layer-4 input as the tensor core saw it)
#pragma unroll
    for (int k = 0; k < 64; k++) h[k] = ld_bf16(sm, PL::HT3 + koff(k, t, 64));
    // dW4 [4][64] and db4 on the CUDA cores
#pragma unroll
    for (int nn = 0; nn < 4; nn++) {
      float v[64];
#pragma unroll
      for (int k = 0; k < 64; k++) v[k] = dO[nn] * h[k];
      warp_reduce_scatter<64>(v, lane);
      const int b = rs_base(lane, 64);
      atomicAdd(&dW4s[nn * 64 + b], v[0]);
      atomicAdd(&dW4s[nn * 64 + b + 1], v[1]);
    }
#pragma unroll
    for (int nn = 0; nn < 4; nn++) {
      float s = dO[nn];
#pragma unroll
      for (int o2 = 16; o2 > 0; o2 >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o2);
      if (lane == 0) atomicAdd(&db4s[nn], s);
    }
    // ---- dX3 = dO W4
    ok = mma_step(mbar, phase, [&] { gemm(tmem, D0, sDO, 128, sW4T, 64, 16, false); });
    if (!ok) break;
    float g[64];
#pragma unroll
    for (int c = 0; c < 4; c++) tmem_ld16(tlane + D0 + 16 * c, g + 16 * c);
#pragma unroll
    for (int k = 0; k < 64; k++) g[k] *= (1.0f - h[k] * h[k]);   // dz3
#pragma unroll
    for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::Q, t, k0, 128, g + k0);
#pragma unroll
    for (int k = 0; k < 64; k++) st_bf16(sm, PL::DZT + koff(k, t, 128), g[k]);
    {
      float v[64];
#pragma unroll
      for (int k = 0; k < 64; k++) v[k] = g[k];
      warp_reduce_scatter<64>(v, lane);
      const int b = rs_base(lane, 64);
      atomicAdd(&db3s[b], v[0]);
      atomicAdd(&db3s[b + 1], v[1]);
    }
    // ---- dX2 = dz3 W3, dW3 += dz3^T H2
    const bool acc = !first;
    ok = mma_step(mbar, phase, [&] {
      gemm(tmem, D0, sQ, 128, sW3T, 64, 64, false);
      gemm(tmem, DW3, sDZT, 128, sHT2, 64, 128, acc);
    });
    if (!ok) break;
#pragma unroll
    for (int c = 0; c < 4; c++) tmem_ld16(tlane + D0 + 16 * c, g + 16 * c);
#pragma unroll
    for (int k = 0; k < 64; k++) {
      const float h2 = ld_bf16(sm, PL::HT2 + koff(k, t, 64));
      g[k] *= (1.0f - h2 * h2);   // dz2
    }
#pragma unroll
    for (int k0 = 0; k0 < 64; k0 += 8) st_row8(sm + PL::P, t, k0, 128, g + k0);
#pragma unroll
    for (int k = 0; k < 64; k++) st_bf16(sm, PL::DZT + koff(k, t, 128), g[k]);
    {
      float v[64];
#pragma unroll
      for (int k = 0; k < 64; k++) v[k] = g[k];
      warp_reduce_scatter<64>(v, lane);
      const int b = rs_base(lane, 64);
      atomicAdd(&db2s[b], v[0]);
      atomicAdd(&db2s[b + 1], v[1]);
    }
    // ---- dX1 = dz2 W2, dW2 += dz2^T H1
    ok = mma_step(mbar, phase, [&] {
      gemm(tmem, D0, sP, 128, sW2T, 64, 64, false);
      gemm(tmem, DW2, sDZT, 128, sHT1, 64, 128, acc);
    });
    if (!ok) break;
#pragma unroll
    for (int c = 0; c < 4; c++) tmem_ld16(tlane + D0 + 16 * c, g + 16 * c);
#pragma unroll
    for (int k = 0; k < 64; k++) {
      const float h1 = ld_bf16(sm, PL::HT1 + koff(k, t, 64));
      g[k] *= (1.0f - h1 * h1);   // dz1
    }
    {
      float v[64];
#pragma unroll
      for (int k = 0; k < 64; k++) v[k] = g[k];
      warp_reduce_scatter<64>(v, lane);
      const int b = rs_base(lane, 64);
      atomicAdd(&db1s[b], v[0]);
      atomicAdd(&db1s[b + 1], v[1]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {   // dW1 [64][4]
      float v[64];
#pragma unroll
      for (int nn = 0; nn < 64; nn++) v[nn] = g[nn] * xb[k];
      warp_reduce_scatter<64>(v, lane);
      const int b = rs_base(lane, 64);
      atomicAdd(&dW1s[b * 4 + k], v[0]);
      atomicAdd(&dW1s[(b + 1) * 4 + k], v[1]);
    }
    first = false;
  }
  if (!ok && t == 0) atomicExch(err, 1);
  // ---- flush: TMEM weight gradients (rows 0..63 = warps 0, 1), CUDA-core sums
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (ok && !first && warp < 2) {
    const int nrow = t;   // output neuron
    float v[64];
#pragma unroll
    for (int c = 0; c < 4; c++) tmem_ld16(tlane + DW2 + 16 * c, v + 16 * c);
#pragma unroll
    for (int k = 0; k < 64; k++) atomicAdd(&grads[kW2 + nrow * 64 + k], v[k]);
#pragma unroll
    for (int c = 0; c < 4; c++) tmem_ld16(tlane + DW3 + 16 * c, v + 16 * c);
#pragma unroll
    for (int k = 0; k < 64; k++) atomicAdd(&grads[kW3 + nrow * 64 + k], v[k]);
  }
  {
    double s = sse;
#pragma unroll
    for (int o2 = 16; o2 > 0; o2 >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o2);
    if (lane == 0) atomicAdd(sse_s, s);
  }
  __syncthreads();
  if (ok && !first) {
    for (int i = t; i < 256; i += blockDim.x) {
      atomicAdd(&grads[kW1 + i], dW1s[i]);
      atomicAdd(&grads[kW4 + i], dW4s[i]);
    }
    for (int i = t; i < 64; i += blockDim.x) {
      atomicAdd(&grads[kB1 + i], db1s[i]);
      atomicAdd(&grads[kB2 + i], db2s[i]);
      atomicAdd(&grads[kB3 + i], db3s[i]);
    }
    if (t < 4) atomicAdd(&grads[kB4 + t], db4s[t]);
    if (t == 0) atomicAdd(sse_out, *sse_s);
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

__global__ void k_mlp_adam(float* prm, const float* __restrict__ g, float* m, float* v, float lr, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float b1 = 0.9f, b2 = 0.999f;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  prm[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

// splitmix64 (Steele, Lea, Flood 2014) as a counter-based generator.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t ctr) {
  return (double)(mix64(seed ^ mix64(ctr)) >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void k_mlp_samples(EosDev eos, int64_t n, uint64_t seed, float* feat, float* tgt, int32_t* ok) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double lo[4], hi[4];
  model_box(eos, M_TABLE, lo, hi);
  double x[4];
  for (int k = 0; k < 4; k++) x[k] = lo[k] + (hi[k] - lo[k]) * uniform01(seed, (uint64_t)i * 4 + k);
  double o[17];
  model_thermo(eos, M_TABLE, x, o);
  const double e = o[5];
  bool good = e > 0.0 && isfinite(e);
  const double ie34 = good ? pow(e, -0.75) : 0.0;
  const double f[4] = {good ? log(e) : 0.0, o[2] * ie34, o[3] * ie34, o[4] * ie34};
  const double y[4] = {log(x[0]), x[1] / x[0], x[2] / x[0], x[3] / x[0]};
  for (int k = 0; k < 4; k++) good = good && isfinite(f[k]);
  for (int k = 0; k < 4; k++) {   // invalid rows carry NaN features: the gradient kernel skips them
    feat[4 * i + k] = good ? (float)f[k] : __int_as_float(0x7fc00000);
    tgt[4 * i + k] = (float)y[k];
  }
  ok[i] = good ? 1 : 0;
}

__global__ void k_mlp_standardise(MlpNorm nm, int64_t n, float* feat, float* tgt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 4; k++) {
    feat[4 * i + k] = (feat[4 * i + k] - nm.in_mean[k]) / nm.in_std[k];
    tgt[4 * i + k] = (tgt[4 * i + k] - nm.out_mean[k]) / nm.out_std[k];
  }
}

}  // namespace

int mlp_smem_forward() { return (int)FwdPlan::BYTES; }
int mlp_smem_grad() { return (int)GradPlan::BYTES; }

namespace {
int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}
}  // namespace

void launch_mlp_forward(const float* params, int64_t n, const float* feat, float* out, int32_t* err, cudaStream_t s) {
  if (n <= 0) return;
  cudaFuncSetAttribute(k_mlp_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FwdPlan::BYTES);
  const int64_t ntiles = (n + kTile - 1) / kTile;
  const int grid = (int)std::min<int64_t>(ntiles, 3 * sm_count());
  k_mlp_fwd<false><<<grid, kTile, FwdPlan::BYTES, s>>>(params, MlpNorm{}, n, feat, out, nullptr, nullptr, err);
}

void launch_mlp_seed(const MlpDev& m, int64_t n, const double* in4, double* tbqs, int32_t* err, cudaStream_t s) {
  if (n <= 0) return;
  cudaFuncSetAttribute(k_mlp_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FwdPlan::BYTES);
  const int64_t ntiles = (n + kTile - 1) / kTile;
  const int grid = (int)std::min<int64_t>(ntiles, 3 * sm_count());
  k_mlp_fwd<true><<<grid, kTile, FwdPlan::BYTES, s>>>(m.params, m.norm, n, nullptr, nullptr, in4, tbqs, err);
}

void launch_mlp_grad(const float* params, int64_t n, const float* feat, const float* tgt, float* grads, double* sse,
                     int32_t* err, cudaStream_t s) {
  if (n <= 0) return;
  cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GradPlan::BYTES);
  const int64_t ntiles = (n + kTile - 1) / kTile;
  const int grid = (int)std::min<int64_t>(ntiles, sm_count());
  k_mlp_grad<<<grid, kTile, GradPlan::BYTES, s>>>(params, n, feat, tgt, grads, sse, err);
}

void launch_mlp_adam(float* params, const float* grads, float* m, float* v, float lr, int t, cudaStream_t s) {
  const float c1 = 1.0f / (1.0f - powf(0.9f, (float)t)), c2 = 1.0f / (1.0f - powf(0.999f, (float)t));
  k_mlp_adam<<<(kParams + 255) / 256, 256, 0, s>>>(params, grads, m, v, lr, c1, c2);
}

void launch_mlp_samples(const EosDev& eos, int64_t n, uint64_t seed, float* feat, float* tgt, int32_t* ok,
                        cudaStream_t s) {
  if (n <= 0) return;
  k_mlp_samples<<<(int)((n + 255) / 256), 256, 0, s>>>(eos, n, seed, feat, tgt, ok);
}

void launch_mlp_standardise(const MlpNorm& nm, int64_t n, float* feat, float* tgt, cudaStream_t s) {
  if (n <= 0) return;
  k_mlp_standardise<<<(int)((n + 255) / 256), 256, 0, s>>>(nm, n, feat, tgt);
}

}  // namespace ccake
