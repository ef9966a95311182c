// Generic compact-operator line kernel for sm_103a.
//
// Every compact operator of the reference (first/second derivatives
// src/derive.f90:7-3792, filters src/filters.f90:221-1377, staggered
// derivatives/interpolations src/derive.f90:3796-5615) has the same shape on
// each grid line:
//     t = A^{-1} (B u)       [+ Sherman-Morrison correction when periodic]
// with B a banded right-hand-side stencil (special rows at the two ends) and A
// tridiagonal with precomputed LU factors (prepare, src/schemes.f90:413-439).
//
// GB300 mapping: one CTA = 32 lines x 16 chunks (512 threads).
//   * The 32 lines' input is staged in shared memory (one coalesced pass over
//     HBM).  For y- and z-lines the 32 lanes are 32 consecutive x-points, so
//     every row is one contiguous 128/256-byte segment; for x-lines the 32
//     lines are consecutive in memory and the tile is transposed on the way in.
//   * Each thread owns one chunk of L = ceil(n/16) rows of one line and keeps
//     them in registers.  The Thomas forward and backward recurrences are run
//     chunk-locally and stitched with a 16-step carry scan through shared
//     memory (fix-up factors pf/qb are data-independent and precomputed), so
//     every element is read once from and written once to HBM.
//   * The periodic Sherman-Morrison vector is precomputed per operator.
#pragma once
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "x3d_internal.h"

namespace x3d {
namespace lk {

constexpr int LANES = 32;
constexpr int CHUNKS = 16;
constexpr int LD = LANES + 1;  // padded tile row (conflict-free transposes)

template <typename T>
struct BRowD {
  T coef[kMaxTerms];
  short idx[kMaxTerms][kMaxEnt];
  signed char mult[kMaxTerms][kMaxEnt];
  signed char nent[kMaxTerms];
  signed char nterms;
  short row;
};

template <typename T>
__device__ __forceinline__ T fuse_out(const Fuse<T>& f, T t, long long i) {
  T o = (f.cr != T(0)) ? f.cr * t : T(0);
  if (f.a1) o = o + f.c1 * f.a1[i];
  if (f.a2) o = o + f.c2 * f.a2[i];
  if (f.y) o = o + f.y[i] * t;
  return o;
}

template <typename T>
struct LineArgs {
  const T* in;
  T* out;
  long long sa_in, sb_in, rs_in, sa_out, sb_out, rs_out;
  int nin, nout, na, L;
  const T *s, *f, *w, *pf, *qb, *rsm, *pp;
  T ca, cb, cc, cd, alpha, den;
  int periodic, nterms_int, nbrows;
  // circulant form of a periodic line (circ = 1): A = (I + mu S)(I + mu S^-1)
  // / (1 + mu^2) with ca..cd pre-scaled by 1 + mu^2; forward / backward
  // recurrences with the constant -mu, chunk fix-ups cpw[k] = (-mu)^(k+1) and
  // cqw[k] = (-mu)^(L-k), cyclic carries from cJ neighbouring chunks with the
  // multiplier cA = (-mu)^L; no Sherman-Morrison pass
  int circ, cJ;
  T cnmu, cA;
  T cpw[32], cqw[32];
  BRowD<T> brows[kMaxBRows];
  Fuse<T> fz;
};

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

template <int KIND>
struct Ext;
template <> struct Ext<K_DER1> { static constexpr int lo = -2, hi = 2; };
template <> struct Ext<K_DER2> { static constexpr int lo = -4, hi = 4; };
template <> struct Ext<K_FIL> { static constexpr int lo = -3, hi = 3; };
template <> struct Ext<K_DVP> { static constexpr int lo = -1, hi = 2; };
template <> struct Ext<K_IVP> { static constexpr int lo = -3, hi = 4; };
template <> struct Ext<K_DPV> { static constexpr int lo = -2, hi = 1; };
template <> struct Ext<K_IPV> { static constexpr int lo = -4, hi = 3; };

// Interior stencil, term order as in the reference's inner loops.
template <typename T, int KIND, typename F>
__device__ __forceinline__ T interior(const F& U, int r, const LineArgs<T>& p) {
  if constexpr (KIND == K_DER1) {
    return p.ca * (U(r + 1) - U(r - 1)) + p.cb * (U(r + 2) - U(r - 2));
  } else if constexpr (KIND == K_DER2) {
    const T ur = U(r);
    T acc = p.ca * (U(r + 1) - ur - ur + U(r - 1)) + p.cb * (U(r + 2) - ur - ur + U(r - 2));
    if (p.nterms_int > 2) acc = acc + p.cc * (U(r + 3) - ur - ur + U(r - 3)) + p.cd * (U(r + 4) - ur - ur + U(r - 4));
    return acc;
  } else if constexpr (KIND == K_FIL) {
    return p.ca * U(r) + p.cb * (U(r + 1) + U(r - 1)) + p.cc * (U(r + 2) + U(r - 2)) + p.cd * (U(r + 3) + U(r - 3));
  } else if constexpr (KIND == K_DVP) {
    return p.ca * (U(r + 1) - U(r)) + p.cb * (U(r + 2) - U(r - 1));
  } else if constexpr (KIND == K_IVP) {
    T acc = p.ca * (U(r + 1) + U(r)) + p.cb * (U(r + 2) + U(r - 1)) + p.cc * (U(r + 3) + U(r - 2));
    if (p.nterms_int > 3) acc = acc + p.cd * (U(r + 4) + U(r - 3));
    return acc;
  } else if constexpr (KIND == K_DPV) {
    return p.ca * (U(r) - U(r - 1)) + p.cb * (U(r + 1) - U(r - 2));
  } else {
    T acc = p.ca * (U(r) + U(r - 1)) + p.cb * (U(r + 1) + U(r - 2)) + p.cc * (U(r + 2) + U(r - 3));
    if (p.nterms_int > 3) acc = acc + p.cd * (U(r + 3) + U(r - 4));
    return acc;
  }
}

template <typename T, int KIND>
__device__ __forceinline__ T rhs_row(const LineArgs<T>& p, const T* tile, int lane, int r) {
  const int nin = p.nin;
  if (r + Ext<KIND>::lo >= 0 && r + Ext<KIND>::hi < nin) {
    auto U = [&](int i) { return tile[i * LD + lane]; };
    return interior<T, KIND>(U, r, p);
  }
  if (p.periodic) {
    auto U = [&](int i) {
      i = (i < 0) ? i + nin : (i >= nin ? i - nin : i);
      return tile[i * LD + lane];
    };
    return interior<T, KIND>(U, r, p);
  }
  // Boundary rows: unfused round-to-nearest operations in the reference's
  // order.  The one-sided closures sum terms of size ~u/dx^2 that cancel, so
  // fusing would change the result well above round-off of the output.
  for (int q = 0; q < p.nbrows; ++q) {
    const BRowD<T>& b = p.brows[q];
    if (b.row != r) continue;
    T acc = T(0);
    for (int t = 0; t < b.nterms; ++t) {
      T v = T(b.mult[t][0]) * tile[b.idx[t][0] * LD + lane];  // mult = +-1, +-2: exact
      for (int e = 1; e < b.nent[t]; ++e) v = add_rn(v, T(b.mult[t][e]) * tile[b.idx[t][e] * LD + lane]);
      acc = (t == 0) ? mul_rn(b.coef[t], v) : add_rn(acc, mul_rn(b.coef[t], v));
    }
    return acc;
  }
  return T(0);
}

template <typename T, int KIND, bool XL, int LMAX, bool CIRC>
__device__ __forceinline__ void line_body(const LineArgs<T>& p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);
  const int nin = p.nin, nout = p.nout;
  const int nmax = nin > nout ? nin : nout;
  T* cfw = tile + (size_t)nmax * LD;
  T* cbw = cfw + CHUNKS * LANES;
  T* ends = cbw + CHUNKS * LANES;

  const int lane = threadIdx.x, ch = threadIdx.y;
  const int a0 = blockIdx.x * LANES;
  const long long b = blockIdx.y;
  const int nl = min(LANES, p.na - a0);

  // 1. stage the input lines
  if (!XL) {
    const int a = a0 + lane;
    const bool ok = lane < nl;
    const long long off = (ok ? (long long)a * p.sa_in : 0) + b * p.sb_in;
    const T* src = p.in + off;
    const T* src2 = p.fz.in2 ? p.fz.in2 + off : nullptr;
    for (int r = ch; r < nin; r += CHUNKS)
      tile[r * LD + lane] = ok ? (src2 ? src[r * p.rs_in] * src2[r * p.rs_in] : src[r * p.rs_in]) : T(0);
  } else {
    const long long off = (long long)a0 * p.sa_in + b * p.sb_in;
    const T* src = p.in + off;
    const T* src2 = p.fz.in2 ? p.fz.in2 + off : nullptr;
    for (int l = ch; l < LANES; l += CHUNKS) {
      if (l < nl) {
        for (int r = lane; r < nin; r += LANES) {
          const long long i = (long long)l * p.sa_in + r;
          tile[r * LD + l] = src2 ? src[i] * src2[i] : src[i];
        }
      } else {
        for (int r = lane; r < nin; r += LANES) tile[r * LD + l] = T(0);
      }
    }
  }
  __syncthreads();

  // 2. right-hand side of this thread's chunk
  const int L = p.L;
  const int r0 = ch * L;
  const int r1 = min(r0 + L, nout);
  T v[LMAX];
#pragma unroll
  for (int k = 0; k < LMAX; ++k) {
    const int r = r0 + k;
    v[k] = (r < r1) ? rhs_row<T, KIND>(p, tile, lane, r) : T(0);
  }

  if constexpr (CIRC) {
    // circulant form: every chunk is full (n = CHUNKS * L)
    T y = T(0);
#pragma unroll
    for (int k = 0; k < LMAX; ++k)
      if (k < L) {
        y = fma_t(p.cnmu, y, v[k]);
        v[k] = y;
      }
    cfw[ch * LANES + lane] = y;
    __syncthreads();
    T cin = T(0);
    for (int j = p.cJ; j >= 1; --j) cin = fma_t(p.cA, cin, cfw[((ch - j) & (CHUNKS - 1)) * LANES + lane]);
#pragma unroll
    for (int k = 0; k < LMAX; ++k)
      if (k < L) v[k] = fma_t(p.cpw[k], cin, v[k]);
    T x = T(0);
#pragma unroll
    for (int k = LMAX - 1; k >= 0; --k)
      if (k < L) {
        x = fma_t(p.cnmu, x, v[k]);
        v[k] = x;
      }
    cbw[ch * LANES + lane] = x;
    __syncthreads();
    cin = T(0);
    for (int j = p.cJ; j >= 1; --j) cin = fma_t(p.cA, cin, cbw[((ch + j) & (CHUNKS - 1)) * LANES + lane]);
#pragma unroll
    for (int k = 0; k < LMAX; ++k)
      if (k < L) v[k] = fma_t(p.cqw[k], cin, v[k]);
  } else {
  // 3. forward elimination: chunk-local, then carry scan + fix-up
  T y = T(0);
#pragma unroll
  for (int k = 0; k < LMAX; ++k) {
    const int r = r0 + k;
    if (r < r1) {
      y = v[k] - p.s[r] * y;
      v[k] = y;
    }
  }
  if (r1 > r0) cfw[ch * LANES + lane] = y;
  __syncthreads();
  {
    T cin = T(0);
    for (int c = 0; c < ch; ++c) {
      const int e = min((c + 1) * L, nout) - 1;
      cin = cfw[c * LANES + lane] + p.pf[e] * cin;
    }
    if (ch > 0) {
#pragma unroll
      for (int k = 0; k < LMAX; ++k) {
        const int r = r0 + k;
        if (r < r1) v[k] = v[k] + p.pf[r] * cin;
      }
    }
  }

  // 4. back substitution: chunk-local, then carry scan + fix-up
  T x = T(0);
#pragma unroll
  for (int k = LMAX - 1; k >= 0; --k) {
    const int r = r0 + k;
    if (r < r1) {
      x = (v[k] - p.f[r] * x) * p.w[r];
      v[k] = x;
    }
  }
  if (r1 > r0) cbw[ch * LANES + lane] = x;
  __syncthreads();
  {
    const int last = (nout - 1) / L;
    T cin = T(0);
    for (int c = last; c > ch; --c) cin = cbw[c * LANES + lane] + p.qb[c * L] * cin;
    if (ch < last) {
#pragma unroll
      for (int k = 0; k < LMAX; ++k) {
        const int r = r0 + k;
        if (r < r1) v[k] = v[k] + p.qb[r] * cin;
      }
    }
  }

  // 5. periodic Sherman-Morrison correction: t -= (t1 - alpha tn)/den * r
  if (p.periodic) {
    if (ch == 0) ends[lane] = v[0];
#pragma unroll
    for (int k = 0; k < LMAX; ++k)
      if (r0 + k < r1 && r0 + k == nout - 1) ends[LANES + lane] = v[k];
    __syncthreads();
    const T sx = (ends[lane] - p.alpha * ends[LANES + lane]) / p.den;
#pragma unroll
    for (int k = 0; k < LMAX; ++k) {
      const int r = r0 + k;
      if (r < r1) v[k] = v[k] - sx * p.rsm[r];
    }
  }
  }  // Thomas form

  if (p.pp) {
#pragma unroll
    for (int k = 0; k < LMAX; ++k) {
      const int r = r0 + k;
      if (r < r1) v[k] = v[k] * p.pp[r];
    }
  }

  // 6. store (with the optional combination epilogue)
  if (!XL) {
    if (lane < nl) {
      const long long off = (long long)(a0 + lane) * p.sa_out + b * p.sb_out;
      T* dst = p.out + off;
#pragma unroll
      for (int k = 0; k < LMAX; ++k) {
        const int r = r0 + k;
        if (r < r1) dst[r * p.rs_out] = p.fz.active ? fuse_out(p.fz, v[k], off + r * p.rs_out) : v[k];
      }
    }
  } else {
    __syncthreads();
#pragma unroll
    for (int k = 0; k < LMAX; ++k) {
      const int r = r0 + k;
      if (r < r1) tile[r * LD + lane] = v[k];
    }
    __syncthreads();
    const long long off = (long long)a0 * p.sa_out + b * p.sb_out;
    T* dst = p.out + off;
    for (int l = ch; l < nl; l += CHUNKS)
      for (int r = lane; r < nout; r += LANES) {
        const long long i = (long long)l * p.sa_out + r;
        dst[i] = p.fz.active ? fuse_out(p.fz, tile[r * LD + l], off + i) : tile[r * LD + l];
      }
  }
}

// Thomas form: the register count is left to the compiler (64 for the
// shorter chunks, two blocks per SM).  Circulant form: one block per SM
// guaranteed, so the long-chunk variant keeps its rows in registers.
template <typename T, int KIND, bool XL, int LMAX>
__global__ void __launch_bounds__(LANES* CHUNKS) line_kernel(const __grid_constant__ LineArgs<T> p) {
  line_body<T, KIND, XL, LMAX, false>(p);
}
template <typename T, int KIND, bool XL, int LMAX>
__global__ void __launch_bounds__(LANES* CHUNKS, 1) line_kernel_circ(const __grid_constant__ LineArgs<T> p) {
  line_body<T, KIND, XL, LMAX, true>(p);
}

template <typename T>
size_t line_smem(int nin, int nout) {
  const int nmax = std::max(nin, nout);
  return sizeof(T) * ((size_t)nmax * LD + 2 * CHUNKS * LANES + 2 * LANES);
}

template <typename T, int KIND, bool XL, int LMAX, bool CIRC = false>
int launch_k(const LineArgs<T>& a, dim3 grid, size_t smem, cudaStream_t st) {
  auto kern = CIRC ? line_kernel_circ<T, KIND, XL, LMAX> : line_kernel<T, KIND, XL, LMAX>;
  static size_t configured = 0;  // largest dynamic smem opted in so far (per instantiation)
  if (smem > configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    configured = smem;
  }
  kern<<<grid, dim3(LANES, CHUNKS), smem, st>>>(a);
  return cuda_status(cudaGetLastError());
}

template <typename T, int KIND>
int dispatch_xl(const LineArgs<T>& a, bool xl, int lmax, dim3 grid, size_t smem, cudaStream_t st) {
  if (a.circ) {
    if (xl) {
      if (lmax == 8) return launch_k<T, KIND, true, 8, true>(a, grid, smem, st);
      if (lmax == 16) return launch_k<T, KIND, true, 16, true>(a, grid, smem, st);
      return launch_k<T, KIND, true, 32, true>(a, grid, smem, st);
    }
    if (lmax == 8) return launch_k<T, KIND, false, 8, true>(a, grid, smem, st);
    if (lmax == 16) return launch_k<T, KIND, false, 16, true>(a, grid, smem, st);
    return launch_k<T, KIND, false, 32, true>(a, grid, smem, st);
  }
  if (xl) {
    if (lmax == 8) return launch_k<T, KIND, true, 8>(a, grid, smem, st);
    if (lmax == 16) return launch_k<T, KIND, true, 16>(a, grid, smem, st);
    return launch_k<T, KIND, true, 32>(a, grid, smem, st);
  }
  if (lmax == 8) return launch_k<T, KIND, false, 8>(a, grid, smem, st);
  if (lmax == 16) return launch_k<T, KIND, false, 16>(a, grid, smem, st);
  return launch_k<T, KIND, false, 32>(a, grid, smem, st);
}

// One translation unit per operator kind instantiates these (x3d_lines_k*.cu).
template <int KIND>
int line_dispatch(const LineArgs<double>& a, bool xl, int lmax, dim3 grid, size_t smem, cudaStream_t st);
template <int KIND>
int line_dispatch(const LineArgs<float>& a, bool xl, int lmax, dim3 grid, size_t smem, cudaStream_t st);

}  // namespace lk
}  // namespace x3d
