// Periodic compact solves in circulant form (binary32), shared by the fused
// line kernels (x3d_conv_diff.cu: momentum right-hand side; x3d_stag_circ.cu:
// staggered divergence / gradient operators).
//
// On a periodic line the compact matrix of every operator here is circulant,
// A = I + alpha (S + S^-1) with S the cyclic shift, and factors exactly as
//   A = (I + mu S)(I + mu S^-1) / (1 + mu^2),  mu = 2 alpha / (1 + sqrt(1 - 4 alpha^2)),
// so x = A^-1 b is a forward recurrence z_i = (1 + mu^2) b_i - mu z_{i-1}
// followed by a backward one x_i = z_i - mu x_{i+1}, both cyclic.  The reference
// solves the same system by Thomas sweeps of a corner-modified matrix plus a
// Sherman-Morrison correction (src/derive.f90:7-64); both give A^-1 b, to
// round-off.  In this form every row has the same coefficients, so a chunk of
// L rows is solved locally from a zero carry and corrected by
//   z_k += (-mu)^(k+1) c_in,      x_k += (-mu)^(L-k) c_in',
// where the carries c_in come from a cyclic scan of the chunk ends with the
// constant multiplier (-mu)^L; terms below binary32 resolution
// ((-mu)^(jL) < 2^-32) are dropped, which is exact to round-off for the
// chunk lengths used (L >= 4, |mu| <= 0.39).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "x3d_line_fast.cuh"

namespace x3d {
namespace lk {

// One periodic compact operator in circulant form (binary32).
struct CircOp {
  float c1, c2, c3, c4;  // interior stencil coefficients times (1 + mu^2)
  float nmu;             // -mu
  int nterms;            // stencil terms: second derivative 2 or 4, interpolation 3 or 4
  int J;                 // chunk carries that reach binary32 (block kernel)
  float Ach;             // (-mu)^L: carry multiplier across one chunk
  float ak[5];           // Ach^(2^s): cyclic warp scan, s = 0..4
  float pw[32];          // (-mu)^(k+1): forward fix-up of chunk row k
  float qw[32];          // (-mu)^(L-k): backward fix-up of chunk row k
};

// Interior stencil (right-hand side B u) on the window w, w[j] = u[r0 - LO + j],
// for every operator kind (the staggered ones map between the velocity and
// the pressure mesh, which coincide in size on a periodic line).
template <int KIND, int LO, typename V>
__device__ __forceinline__ V circ_rhs_t(const V* w, int k, const CircOp& p) {
#define W_(d) w[k + LO + (d)]
  if constexpr (KIND == K_DER1) {
    return p.c1 * (W_(1) - W_(-1)) + p.c2 * (W_(2) - W_(-2));
  } else if constexpr (KIND == K_DER2) {
    const V ur = W_(0);
    V acc = p.c1 * (W_(1) - ur - ur + W_(-1)) + p.c2 * (W_(2) - ur - ur + W_(-2));
    if (p.nterms > 2) acc = acc + p.c3 * (W_(3) - ur - ur + W_(-3)) + p.c4 * (W_(4) - ur - ur + W_(-4));
    return acc;
  } else if constexpr (KIND == K_FIL) {
    return p.c1 * W_(0) + p.c2 * (W_(1) + W_(-1)) + p.c3 * (W_(2) + W_(-2)) + p.c4 * (W_(3) + W_(-3));
  } else if constexpr (KIND == K_DVP) {
    return p.c1 * (W_(1) - W_(0)) + p.c2 * (W_(2) - W_(-1));
  } else if constexpr (KIND == K_IVP) {
    V acc = p.c1 * (W_(1) + W_(0)) + p.c2 * (W_(2) + W_(-1)) + p.c3 * (W_(3) + W_(-2));
    if (p.nterms > 3) acc = acc + p.c4 * (W_(4) + W_(-3));
    return acc;
  } else if constexpr (KIND == K_DPV) {
    return p.c1 * (W_(0) - W_(-1)) + p.c2 * (W_(1) - W_(-2));
  } else {
    V acc = p.c1 * (W_(0) + W_(-1)) + p.c2 * (W_(1) + W_(-2)) + p.c3 * (W_(2) + W_(-3));
    if (p.nterms > 3) acc = acc + p.c4 * (W_(3) + W_(-4));
    return acc;
  }
#undef W_
}
template <int KIND, int LO>
__device__ __forceinline__ float circ_rhs(const float* w, int k, const CircOp& p) {
  return circ_rhs_t<KIND, LO, float>(w, k, p);
}

// Warp-per-line solve: lane t owns rows t*L .. t*L+L-1 of a 32*L line; the
// chunk carries are an inclusive cyclic Kogge-Stone scan over the lanes.
template <int KIND, int L>
__device__ __forceinline__ void circ_warp(const float* w, float* v, const CircOp& p, int lane) {
  constexpr int LO = Halo<KIND>::lo;
  constexpr unsigned FULL = 0xffffffffu;
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = circ_rhs<KIND, LO>(w, k, p);
#pragma unroll
  for (int k = 1; k < L; ++k) v[k] = fmaf(p.nmu, v[k - 1], v[k]);
  float b = v[L - 1];
#pragma unroll
  for (int s = 0; s < 5; ++s) b = fmaf(p.ak[s], __shfl_sync(FULL, b, (lane - (1 << s)) & 31), b);
  const float cf = __shfl_sync(FULL, b, (lane + 31) & 31);
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = fmaf(p.pw[k], cf, v[k]);
#pragma unroll
  for (int k = L - 2; k >= 0; --k) v[k] = fmaf(p.nmu, v[k + 1], v[k]);
  b = v[0];
#pragma unroll
  for (int s = 0; s < 5; ++s) b = fmaf(p.ak[s], __shfl_sync(FULL, b, (lane + (1 << s)) & 31), b);
  const float cb = __shfl_sync(FULL, b, (lane + 1) & 31);
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = fmaf(p.qw[k], cb, v[k]);
}

// Asynchronous 4-byte global -> shared copy (LDGSTS): the copies are in
// flight together and hold no registers.
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// Per-warp line buffer of the x kernels: rows -4 .. 32L+3 of a 32L line, row
// r at P(r + L), P(s) = s + floor(s / L) (each lane's window at compile-time
// offsets from one base, lanes L+1 words apart: free of bank conflicts).
template <int L>
__host__ __device__ constexpr int xbuf() {
  return 32 * L + L + 40;
}
template <int L>
__device__ __forceinline__ constexpr int hoff(int d) {
  return d + (d >= 0 ? d / L : -1);  // -L <= d < 2L
}

constexpr int YL = 8;     // rows per chunk
constexpr int CP = 8;     // column pairs per block
constexpr int SR2 = 18;   // slab row stride (floats)

__device__ __forceinline__ float2 f2fma(float a, float2 b, float2 c) {
  return make_float2(fmaf(a, b.x, c.x), fmaf(a, b.y, c.y));
}
__device__ __forceinline__ float2 f2fma2(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
}

// float2 arithmetic for the two-lines-per-thread kernels (component-wise, in
// the same order as the scalar form).
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 operator*(float a, float2 b) { return make_float2(a * b.x, a * b.y); }

template <int KIND, int LO>
__device__ __forceinline__ float2 circ_rhs2(const float2* w, int k, const CircOp& p) {
  return circ_rhs_t<KIND, LO, float2>(w, k, p);
}

// Block solve of two lines per thread: thread (cp, ch) owns rows ch*L ..
// ch*L+L-1 of lines 2cp and 2cp+1; FC chunks per line, carries through shared
// memory (ef / eb: [FC][CP] float2).  Two block barriers; every thread of the
// block must call it.
template <int KIND, int L, int FC>
__device__ __forceinline__ void circ_block2(const float2* w, float2* v, const CircOp& p, float2* ef, float2* eb,
                                            int ch, int cp) {
  constexpr int LO = Halo<KIND>::lo;
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = circ_rhs2<KIND, LO>(w, k, p);
#pragma unroll
  for (int k = 1; k < L; ++k) v[k] = f2fma(p.nmu, v[k - 1], v[k]);
  ef[ch * CP + cp] = v[L - 1];
  __syncthreads();
  float2 c = make_float2(0.f, 0.f);
  for (int j = p.J; j >= 1; --j) c = f2fma(p.Ach, c, ef[((ch - j) & (FC - 1)) * CP + cp]);
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = f2fma2(make_float2(p.pw[k], p.pw[k]), c, v[k]);
#pragma unroll
  for (int k = L - 2; k >= 0; --k) v[k] = f2fma(p.nmu, v[k + 1], v[k]);
  eb[ch * CP + cp] = v[0];
  __syncthreads();
  c = make_float2(0.f, 0.f);
  for (int j = p.J; j >= 1; --j) c = f2fma(p.Ach, c, eb[((ch + j) & (FC - 1)) * CP + cp]);
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = f2fma2(make_float2(p.qw[k], p.qw[k]), c, v[k]);
}

__device__ __forceinline__ void cp_async8(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

// Circulant form of a periodic plan for chunks of L rows (x3d_conv_diff.cu);
// max_carries bounds the carries a block kernel adds.  X3D_ERR_UNSUPPORTED
// for a non-periodic plan or a matrix that is not diagonally dominant.
int fill_circ(const OpPlan* p, int L, int max_carries, CircOp& c);

}  // namespace lk
}  // namespace x3d
