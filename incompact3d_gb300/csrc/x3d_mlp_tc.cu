// Tensor-core inference of the learned SGS closure (10 -> 64 -> 64 -> 6,
// GELU) on the 5th-generation tensor cores: tcgen05.mma with the accumulators
// in tensor memory, weights brought into shared memory by one bulk async copy.
//
// Tile: 128 points = the M of one MMA; thread t of the 4-warp CTA owns point t
// (row t of every operand and TMEM lane t).  Per tile:
//   features -> BF16 hi / lo rows of A (K = 16: 10 features + 6 zeros)
//   layer 1: D[:, 0:64)   = A Wh1^T + A_h Wl1^T + A_l Wh1^T      (3 MMAs)
//   GELU(D + b1) -> hi / lo rows of A (K = 64), same shared buffer
//   layer 2: D[:, 64:128) = same split, 4 K-steps of 16         (12 MMAs)
//   GELU(D + b2) -> A
//   layer 3: D[:, 0:16)   = the 6 outputs (+ 10 zero rows of W3)  (12 MMAs)
// The split product hi*hi + hi*lo + lo*hi of BF16 parts (each value x carried
// as bf16(x) + bf16(x - bf16(x)), 16 significant bits) accumulated in FP32
// keeps the result within a few 2^-16 of the FP32 CUDA-core kernel.
//
// Operand layout in shared memory (no swizzle, K-major): the 8-row x 16-byte
// core matrices of a row group are contiguous along K, so for a matrix of K
// columns element (r, k) sits at byte
//   (r / 8) * 16 K + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. core matrices 128 B apart along K (leading byte offset) and 16 K bytes
// apart along M / N (stride byte offset).  A thread writes its row as 16-byte
// stores, 8 consecutive rows of a warp filling one 128-byte line.
//
// Every wait is bounded (iterations and clock): on expiry the CTA sets *err,
// stops issuing, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "x3d_internal.h"

namespace x3d {
namespace {

using namespace mlpdim;

constexpr int TC_M = 128;                       // points per tile
constexpr int A_BYTES = TC_M * NH * 2;          // one BF16 part of A (K = 64)
constexpr int OFF_AH = 0, OFF_AL = A_BYTES;     // A hi / lo
constexpr int OFF_W = 2 * A_BYTES;              // packed weights
// packed weight image, bytes: W1 (64 x 16) hi, lo; W2 (64 x 64) hi, lo; W3 (16 x 64) hi, lo
constexpr int W1H = 0, W1L = 2048, W2H = 4096, W2L = 12288, W3H = 20480, W3L = 22528;
static_assert(W3L + 2048 == MLP_TC_WP_BYTES, "weight image size");
constexpr int OFF_F = OFF_W + MLP_TC_WP_BYTES;  // b1[64] b2[64] b3[16] insc[16] outsc[8] (floats)
constexpr int NF = 168;
constexpr int OFF_BAR = OFF_F + 4 * NF;         // two mbarriers
constexpr int OFF_SLOT = OFF_BAR + 16;          // tensor-memory address written by tcgen05.alloc
constexpr int TC_SMEM = OFF_SLOT + 16;
static_assert(OFF_BAR % 8 == 0, "mbarrier alignment");
constexpr int TMEM_COLS = 128;                  // layer-1 / layer-3 D in 0..63, layer-2 D in 64..127
constexpr int TC_CTAS_PER_SM = 3;               // 3 x 128 TMEM columns <= 512

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- shared-memory matrix descriptor (tcgen05, no swizzle) ------------------
// bits 0-13 start >> 4, 16-29 leading byte offset >> 4, 32-45 stride byte
// offset >> 4, bit 46 the fixed descriptor version 1, 61-63 swizzle 0.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: about one second of SM clock or 2^22 polls, whichever first.
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  for (int i = 0; i < (1 << 22); ++i) {
    if (mbar_try(bar, parity)) return true;
    if (clock64() - t0 > 2000000000ll) break;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }

// BF16 hi / lo parts of two values packed as the 32-bit words of a row.
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Row r, 16 values v (K positions 16 g .. 16 g + 15) of a K-column operand.
template <int K>
__device__ __forceinline__ void store16(uint8_t* sm, int r, int g, const float* v) {
  uint32_t h[8], l[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) split2(v[2 * j], v[2 * j + 1], h[j], l[j]);
  const int o = (r >> 3) * (16 * K) + (2 * g) * 128 + (r & 7) * 16;
  *reinterpret_cast<uint4*>(sm + OFF_AH + o) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(sm + OFF_AH + o + 128) = make_uint4(h[4], h[5], h[6], h[7]);
  *reinterpret_cast<uint4*>(sm + OFF_AL + o) = make_uint4(l[0], l[1], l[2], l[3]);
  *reinterpret_cast<uint4*>(sm + OFF_AL + o + 128) = make_uint4(l[4], l[5], l[6], l[7]);
}

// One K-step of 16 of the split product into TMEM column d.
__device__ __forceinline__ void mma_split(uint32_t d, uint32_t ah, uint32_t al, uint32_t wh, uint32_t wl,
                                          uint32_t sbo_a, uint32_t sbo_w, uint32_t id, bool first) {
  mma_bf16(d, sdesc(ah, 128, sbo_a), sdesc(wh, 128, sbo_w), id, first ? 0u : 1u);
  mma_bf16(d, sdesc(ah, 128, sbo_a), sdesc(wl, 128, sbo_w), id, 1u);
  mma_bf16(d, sdesc(al, 128, sbo_a), sdesc(wh, 128, sbo_w), id, 1u);
}

struct TcArgs {
  const float* P;
  const float* sc;
  const void* wp;
  int* err;
  const float* X;
  float* Y;
  const double* g[9];
  double* tau[6];
  float delta;
  long long n;
};

__global__ void __launch_bounds__(TC_M, TC_CTAS_PER_SM) k_mlp_tc(const __grid_constant__ TcArgs a) {
  extern __shared__ __align__(128) uint8_t sm[];
  float* fb = reinterpret_cast<float*>(sm + OFF_F);
  float *b1 = fb, *b2 = fb + 64, *b3 = fb + 128, *insc = fb + 144, *outsc = fb + 160;
  const int t = threadIdx.x, warp = t >> 5;
  const uint32_t s0 = smem_u32(sm);
  const uint32_t bar_w = s0 + OFF_BAR, bar_m = s0 + OFF_BAR + 8;
  const uint32_t ah = s0 + OFF_AH, al = s0 + OFF_AL, w = s0 + OFF_W;

  if (t == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_m, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (t < 64) {
    b1[t] = a.P[OB1 + t];
    b2[t] = a.P[OB2 + t];
  }
  if (t < 16) {
    b3[t] = t < NO ? a.P[OB3 + t] : 0.f;
    insc[t] = t < NI ? a.sc[t] : 0.f;
  }
  if (t < 8) outsc[t] = t < NO ? a.sc[NI + t] : 0.f;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s0 + OFF_SLOT),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + OFF_SLOT);
  const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's 32 TMEM lanes

  if (t == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_w), "r"(MLP_TC_WP_BYTES)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(w),
        "l"(a.wp), "r"(MLP_TC_WP_BYTES), "r"(bar_w)
        : "memory");
  }
  int bad = __syncthreads_or(!mbar_wait(bar_w, 0));
  uint32_t ph = 0;
  int pend = -1;  // thread 0: parity of an MMA commit whose completion it has not seen
  const long long ntiles = (a.n + TC_M - 1) / TC_M;
  constexpr uint32_t ID64 = idesc_bf16(TC_M, 64), ID16 = idesc_bf16(TC_M, 16);

  for (long long tile = blockIdx.x; tile < ntiles && !bad; tile += gridDim.x) {
    const long long m = tile * TC_M + t;
    const bool live = m < a.n;
    {  // features -> A (K = 16)
      float x[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) x[i] = 0.f;
      if (live) {
        if (a.X) {
#pragma unroll
          for (int i = 0; i < NI; ++i) x[i] = a.X[m * NI + i] * insc[i];
        } else {
#pragma unroll
          for (int i = 0; i < 9; ++i) x[i] = (float)a.g[i][m] * insc[i];
          x[9] = a.delta * insc[9];
        }
      }
      store16<16>(sm, t, 0, x);
    }
    proxy_fence();
    __syncthreads();
    if (t == 0) {
      tc_after();
      mma_split(tmem, ah, al, w + W1H, w + W1L, 256, 256, ID64, true);
      mma_commit(bar_m);
    }
    bad = !mbar_wait(bar_m, ph);
    if (bad && t == 0) pend = (int)ph;
    ph ^= 1;
    tc_after();
    // layer-1 epilogue: H1 = GELU(D + b1) -> A (K = 64); the MMAs reading A are done
#pragma unroll 1
    for (int g = 0; g < 4; ++g) {
      float v[16];
      tmem_ld16(trow + 16 * g, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = gelu(v[j] + b1[16 * g + j]);
      store16<64>(sm, t, g, v);
    }
    proxy_fence();
    tc_before();
    if ((bad = __syncthreads_or(bad))) break;
    if (t == 0) {
      tc_after();
#pragma unroll
      for (int s = 0; s < 4; ++s)
        mma_split(tmem + 64, ah + 256 * s, al + 256 * s, w + W2H + 256 * s, w + W2L + 256 * s, 1024, 1024, ID64,
                  s == 0);
      mma_commit(bar_m);
    }
    bad = !mbar_wait(bar_m, ph);
    if (bad && t == 0) pend = (int)ph;
    ph ^= 1;
    tc_after();
#pragma unroll 1
    for (int g = 0; g < 4; ++g) {
      float v[16];
      tmem_ld16(trow + 64 + 16 * g, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = gelu(v[j] + b2[16 * g + j]);
      store16<64>(sm, t, g, v);
    }
    proxy_fence();
    tc_before();
    if ((bad = __syncthreads_or(bad))) break;
    if (t == 0) {
      tc_after();
#pragma unroll
      for (int s = 0; s < 4; ++s)
        mma_split(tmem, ah + 256 * s, al + 256 * s, w + W3H + 256 * s, w + W3L + 256 * s, 1024, 1024, ID16, s == 0);
      mma_commit(bar_m);
    }
    bad = !mbar_wait(bar_m, ph);
    if (bad && t == 0) pend = (int)ph;
    ph ^= 1;
    tc_after();
    {
      float v[16];
      tmem_ld16(trow, v);
      if (live) {
        if (a.Y) {
#pragma unroll
          for (int q = 0; q < NO; ++q) a.Y[m * NO + q] = (v[q] + b3[q]) * outsc[q];
        } else {
#pragma unroll
          for (int q = 0; q < NO; ++q) a.tau[q][m] = (double)((v[q] + b3[q]) * outsc[q]);
        }
      }
    }
    tc_before();
    bad = __syncthreads_or(bad);
  }
  if (bad) {
    // a weight copy still in flight is waited for (bounded) before the CTA exits,
    // and so is an MMA group whose completion was not seen, before its
    // tensor memory is freed
    if (t == 0) {
      mbar_wait(bar_w, 0);
      if (pend >= 0) mbar_wait(bar_m, (uint32_t)pend);
      atomicExch(a.err, 1);
    }
  }
  tc_before();
  __syncthreads();
  tc_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// BF16 hi / lo image of W1 (64 x 16, inputs 10..15 zero), W2 (64 x 64) and W3
// (16 x 64, outputs 6..15 zero) in the operand layout above.
__global__ void k_mlp_tc_pack(const float* P, uint16_t* out) {
  const int nel = 64 * 16 + 64 * 64 + 16 * 64;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nel; i += gridDim.x * blockDim.x) {
    int R, K, r, k, off;
    float v;
    if (i < 1024) {
      R = 64, K = 16, r = i / 16, k = i % 16, off = W1H / 2;
      v = k < NI ? P[OW1 + r * NI + k] : 0.f;
    } else if (i < 1024 + 4096) {
      const int j = i - 1024;
      R = 64, K = 64, r = j / 64, k = j % 64, off = W2H / 2;
      v = P[OW2 + r * NH + k];
    } else {
      const int j = i - 5120;
      R = 16, K = 64, r = j / 64, k = j % 64, off = W3H / 2;
      v = r < NO ? P[OW3 + r * NH + k] : 0.f;
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
    const int e = (r >> 3) * (8 * K) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
    out[off + e] = *reinterpret_cast<const uint16_t*>(&h);
    out[off + R * K + e] = *reinterpret_cast<const uint16_t*>(&l);
  }
}

}  // namespace

int mlp_tc_pack(const float* P, void* wp, cudaStream_t st) {
  k_mlp_tc_pack<<<24, 256, 0, st>>>(P, static_cast<uint16_t*>(wp));
  return cuda_status(cudaGetLastError());
}

int mlp_tc_infer(const float* P, const float* sc, const void* wp, int* err, const float* X, float* Y,
                 const double* const* g9, float delta, double* const* tau6, long long n, int num_sms,
                 cudaStream_t st) {
  if (n <= 0) return X3D_OK;
  if ((reinterpret_cast<uintptr_t>(wp) & 15) != 0) return X3D_ERR_ARG;
  TcArgs a{};
  a.P = P;
  a.sc = sc;
  a.wp = wp;
  a.err = err;
  a.X = X;
  a.Y = Y;
  if (!X) {
    for (int i = 0; i < 9; ++i) a.g[i] = g9[i];
    for (int i = 0; i < 6; ++i) a.tau[i] = tau6[i];
  }
  a.delta = delta;
  a.n = n;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  const long long ntiles = (n + TC_M - 1) / TC_M;
  const long long grid = std::min<long long>(ntiles, (long long)num_sms * TC_CTAS_PER_SM);
  k_mlp_tc<<<(unsigned)grid, TC_M, TC_SMEM, st>>>(a);
  return cuda_status(cudaGetLastError());
}

}  // namespace x3d
