// Fast path of the compact-operator line kernel for periodic lines whose
// length is 16*L (L = 8, 16 or 32): every chunk is full, so nothing is
// predicated.  Same algorithm as line_kernel (x3d_line_kernel.cuh) with a
// leaner instruction stream:
//   * y/z lines: each thread loads its chunk plus the stencil halo straight
//     from HBM into a register window (32 consecutive x-points per warp: one
//     coalesced 128-byte row segment per load); no shared-memory tile.
//     x lines: the 32 lines are staged once through a padded shared tile (the
//     transpose), then read into the same register window.
//   * away from the line ends the LU factors are constant to the last bit
//     (the pivots of prepare() converge), so those chunks use three scalar
//     factors and generate the chunk fix-up factors by running products
//     instead of loading six coefficient vectors per row;
//   * the Sherman-Morrison correction is applied only to chunks where the
//     precomputed vector is non-zero in this precision.
// The chunk solve is a device function (fast_solve) so that one kernel can
// run several operators on the same lines (the momentum right-hand
// side: three solves per line, one HBM pass per input field).
#pragma once
#include "x3d_line_kernel.cuh"

namespace x3d {
namespace lk {

constexpr int FCHUNKS = 16;

// Coefficients of one operator for the fast path.
template <typename T>
struct FastOp {
  const T *s, *f, *w, *pf, *qb, *rsm;  // per-row vectors (non-uniform chunks)
  T ca, cb, cc, cd, alpha, den;
  T s_inf, f_inf, w_inf, g_inf;  // interior factors; g = -(f*w)
  T pfe[FCHUNKS];                // pf at each chunk's last row
  T qbs[FCHUNKS];                // qb at each chunk's first row
  int mode[FCHUNKS];             // bit0: uniform factors, bit1: SM vector non-zero
  int nterms_int;
  T pw[32];                      // uniform chunks: forward fix-up (-s)^(k+1)
  T qw[32];                      // uniform chunks: backward fix-up g^(L-k)
};

template <typename T>
struct FastArgs {
  const T* in;
  T* out;
  long long sa, sb, rs;  // line (a, b) offset and row stride (same for in and out)
  int n, na;
  FastOp<T> op;
  Fuse<T> fz;  // optional product on load / combination on store
};

template <int KIND>
struct Halo {
  static constexpr int lo = -Ext<KIND>::lo, hi = Ext<KIND>::hi;
};

// Interior stencil on the register window: w[j] holds u[r0 - lo + j].
template <typename T, int KIND, int LO>
__device__ __forceinline__ T interior_w(const T* w, int k, const FastOp<T>& p) {
#define W_(d) w[k + LO + (d)]
  if constexpr (KIND == K_DER1) {
    return p.ca * (W_(1) - W_(-1)) + p.cb * (W_(2) - W_(-2));
  } else if constexpr (KIND == K_DER2) {
    const T ur = W_(0);
    T acc = p.ca * (W_(1) - ur - ur + W_(-1)) + p.cb * (W_(2) - ur - ur + W_(-2));
    if (p.nterms_int > 2) acc = acc + p.cc * (W_(3) - ur - ur + W_(-3)) + p.cd * (W_(4) - ur - ur + W_(-4));
    return acc;
  } else if constexpr (KIND == K_FIL) {
    return p.ca * W_(0) + p.cb * (W_(1) + W_(-1)) + p.cc * (W_(2) + W_(-2)) + p.cd * (W_(3) + W_(-3));
  } else if constexpr (KIND == K_DVP) {
    return p.ca * (W_(1) - W_(0)) + p.cb * (W_(2) - W_(-1));
  } else if constexpr (KIND == K_IVP) {
    T acc = p.ca * (W_(1) + W_(0)) + p.cb * (W_(2) + W_(-1)) + p.cc * (W_(3) + W_(-2));
    if (p.nterms_int > 3) acc = acc + p.cd * (W_(4) + W_(-3));
    return acc;
  } else if constexpr (KIND == K_DPV) {
    return p.ca * (W_(0) - W_(-1)) + p.cb * (W_(1) - W_(-2));
  } else {
    T acc = p.ca * (W_(0) + W_(-1)) + p.cb * (W_(1) + W_(-2)) + p.cc * (W_(2) + W_(-3));
    if (p.nterms_int > 3) acc = acc + p.cd * (W_(3) + W_(-4));
    return acc;
  }
#undef W_
}

// Row index of window slot j of chunk ch (periodic wrap only in the first and
// last chunk, whose halos cross the line ends).
__device__ __forceinline__ int wrow(int r, int n, bool edge) {
  return edge ? ((r < 0) ? r + n : (r >= n ? r - n : r)) : r;
}

// Register window of a y/z line from global memory: w[j] = u[r0m + j]
// (times u2 when given), rows wrapped only in the edge chunks.  Lanes past
// the last line read a
// valid line instead (their results are never stored, and the chunk carries
// are per lane).
template <typename T, int WN>
__device__ __forceinline__ void load_window(T* w, const T* src, const T* src2, int r0m, int n, long long rs,
                                            bool edge) {
  if (src2) {
#pragma unroll
    for (int j = 0; j < WN; ++j) {
      const long long o = (long long)wrow(r0m + j, n, edge) * rs;
      w[j] = src[o] * src2[o];
    }
  } else {
#pragma unroll
    for (int j = 0; j < WN; ++j) w[j] = src[(long long)wrow(r0m + j, n, edge) * rs];
  }
}

// Solve of this thread's chunk (rows ch*L .. ch*L+L-1) of one line:
// v = A^{-1} (B u) with u in the register window w (w[j] = u[r0 - LO + j]).
// Uses the block's carry arrays and three block barriers; every thread of
// the block must call it.
template <typename T, int KIND, int L>
__device__ __forceinline__ void fast_solve(const T* w, T* v, const FastOp<T>& p, T* cfw, T* cbw, T* ends, int ch,
                                           int lane) {
  constexpr int LO = Halo<KIND>::lo;
  const int r0 = ch * L;
  const int mode = p.mode[ch];
  // right-hand side
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = interior_w<T, KIND, LO>(w, k, p);
  // forward elimination + carry scan + fix-up
  T y = T(0);
  if (mode & 1) {
#pragma unroll
    for (int k = 0; k < L; ++k) { y = v[k] - p.s_inf * y; v[k] = y; }
  } else {
#pragma unroll
    for (int k = 0; k < L; ++k) { y = v[k] - p.s[r0 + k] * y; v[k] = y; }
  }
  cfw[ch * LANES + lane] = y;
  __syncthreads();
  if (ch > 0) {
    T cin = T(0);
    for (int c = 0; c < ch; ++c) cin = cfw[c * LANES + lane] + p.pfe[c] * cin;
    if (mode & 1) {
#pragma unroll
      for (int k = 0; k < L; ++k) v[k] = v[k] + p.pw[k] * cin;
    } else {
#pragma unroll
      for (int k = 0; k < L; ++k) v[k] = v[k] + p.pf[r0 + k] * cin;
    }
  }
  // back substitution + carry scan + fix-up
  T x = T(0);
  if (mode & 1) {
#pragma unroll
    for (int k = L - 1; k >= 0; --k) { x = (v[k] - p.f_inf * x) * p.w_inf; v[k] = x; }
  } else {
#pragma unroll
    for (int k = L - 1; k >= 0; --k) { x = (v[k] - p.f[r0 + k] * x) * p.w[r0 + k]; v[k] = x; }
  }
  cbw[ch * LANES + lane] = x;
  __syncthreads();
  if (ch < FCHUNKS - 1) {
    T cin = T(0);
    for (int c = FCHUNKS - 1; c > ch; --c) cin = cbw[c * LANES + lane] + p.qbs[c] * cin;
    if (mode & 1) {
#pragma unroll
      for (int k = 0; k < L; ++k) v[k] = v[k] + p.qw[k] * cin;
    } else {
#pragma unroll
      for (int k = 0; k < L; ++k) v[k] = v[k] + p.qb[r0 + k] * cin;
    }
  }
  // Sherman-Morrison
  if (ch == 0) ends[lane] = v[0];
  if (ch == FCHUNKS - 1) ends[LANES + lane] = v[L - 1];
  __syncthreads();
  if (mode & 2) {
    const T sx = (ends[lane] - p.alpha * ends[LANES + lane]) / p.den;
#pragma unroll
    for (int k = 0; k < L; ++k) v[k] = v[k] - sx * p.rsm[r0 + k];
  }
}

template <typename T, int KIND, bool XL, int L>
__global__ void __launch_bounds__(LANES* FCHUNKS, 2) line_fast(const __grid_constant__ FastArgs<T> p) {
  constexpr int LO = Halo<KIND>::lo, HI = Halo<KIND>::hi;
  constexpr int WN = L + LO + HI;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* cfw = reinterpret_cast<T*>(smem_raw);
  T* cbw = cfw + FCHUNKS * LANES;
  T* ends = cbw + FCHUNKS * LANES;
  T* tile = ends + 2 * LANES;  // x lines only: [n][LD]

  const int lane = threadIdx.x, ch = threadIdx.y;
  const int n = p.n;
  const int a0 = blockIdx.x * LANES;
  const long long b = blockIdx.y;
  const int nl = min(LANES, p.na - a0);
  const int r0 = ch * L;
  const bool edge = (ch == 0 || ch == FCHUNKS - 1);

  // 1. register window u[r0-LO .. r0+L+HI) (periodic wrap)
  T w[WN];
  if (!XL) {
    const bool ok = lane < nl;
    const long long off = (ok ? (long long)(a0 + lane) * p.sa : 0) + b * p.sb;
    load_window<T, WN>(w, p.in + off, p.fz.in2 ? p.fz.in2 + off : nullptr, r0 - LO, n, p.rs, edge);
  } else {
    const long long off = (long long)a0 * p.sa + b * p.sb;
    const T* src = p.in + off;
    const T* src2 = p.fz.in2 ? p.fz.in2 + off : nullptr;
    for (int l = ch; l < LANES; l += FCHUNKS) {
      if (l < nl) {
        if (src2) {
          for (int r = lane; r < n; r += LANES)
            tile[r * LD + l] = src[(long long)l * p.sa + r] * src2[(long long)l * p.sa + r];
        } else {
          for (int r = lane; r < n; r += LANES) tile[r * LD + l] = src[(long long)l * p.sa + r];
        }
      } else {
        for (int r = lane; r < n; r += LANES) tile[r * LD + l] = T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < WN; ++j) w[j] = tile[wrow(r0 - LO + j, n, edge) * LD + lane];
  }

  // 2-5. solve
  T v[L];
  fast_solve<T, KIND, L>(w, v, p.op, cfw, cbw, ends, ch, lane);

  // 6. store (with the optional combination epilogue)
  if (!XL) {
    if (lane < nl) {
      const long long off = (long long)(a0 + lane) * p.sa + b * p.sb;
      T* dst = p.out + off;
      if (p.fz.active) {
        // operands are read in groups of 4 rows before any store of the group:
        // the output may alias a1/a2, so the compiler cannot batch them itself
        constexpr int G = 4;
#pragma unroll
        for (int k0 = 0; k0 < L; k0 += G) {
          T A1[G], A2[G], Y[G];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const long long i = off + (long long)(r0 + k0 + g) * p.rs;
            A1[g] = p.fz.a1 ? p.fz.a1[i] : T(0);
            A2[g] = p.fz.a2 ? p.fz.a2[i] : T(0);
            Y[g] = p.fz.y ? p.fz.y[i] : T(0);
          }
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const T t = v[k0 + g];
            T o = (p.fz.cr != T(0)) ? p.fz.cr * t : T(0);
            o = o + p.fz.c1 * A1[g];
            o = o + p.fz.c2 * A2[g];
            o = o + Y[g] * t;
            dst[(long long)(r0 + k0 + g) * p.rs] = o;
          }
        }
      } else {
#pragma unroll
        for (int k = 0; k < L; ++k) dst[(long long)(r0 + k) * p.rs] = v[k];
      }
    }
  } else {
    __syncthreads();
#pragma unroll
    for (int k = 0; k < L; ++k) tile[(r0 + k) * LD + lane] = v[k];
    __syncthreads();
    const long long off = (long long)a0 * p.sa + b * p.sb;
    T* dst = p.out + off;
    if (p.fz.active) {
      for (int l = ch; l < nl; l += FCHUNKS)
        for (int r = lane; r < n; r += LANES) {
          const long long i = (long long)l * p.sa + r;
          dst[i] = fuse_out(p.fz, tile[r * LD + l], off + i);
        }
    } else {
      for (int l = ch; l < nl; l += FCHUNKS)
        for (int r = lane; r < n; r += LANES) dst[(long long)l * p.sa + r] = tile[r * LD + l];
    }
  }
}

template <typename T>
size_t fast_smem(int n, bool xl) {
  return sizeof(T) * ((size_t)2 * FCHUNKS * LANES + 2 * LANES + (xl ? (size_t)n * LD : 0));
}

template <typename T, int KIND, bool XL, int L>
int launch_fast_k(const FastArgs<T>& a, dim3 grid, size_t smem, cudaStream_t st) {
  auto kern = line_fast<T, KIND, XL, L>;
  static size_t configured = 0;
  if (smem > configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    configured = smem;
  }
  kern<<<grid, dim3(LANES, FCHUNKS), smem, st>>>(a);
  return cuda_status(cudaGetLastError());
}

template <typename T, int KIND>
int fast_dispatch_xl(const FastArgs<T>& a, bool xl, int L, dim3 grid, size_t smem, cudaStream_t st) {
  if (xl) {
    if (L == 8) return launch_fast_k<T, KIND, true, 8>(a, grid, smem, st);
    if (L == 16) return launch_fast_k<T, KIND, true, 16>(a, grid, smem, st);
    return launch_fast_k<T, KIND, true, 32>(a, grid, smem, st);
  }
  if (L == 8) return launch_fast_k<T, KIND, false, 8>(a, grid, smem, st);
  if (L == 16) return launch_fast_k<T, KIND, false, 16>(a, grid, smem, st);
  return launch_fast_k<T, KIND, false, 32>(a, grid, smem, st);
}

// Fast-path coefficients of a periodic FP32 plan, and the line geometry of an
// axis (x3d_lines.cu).
void fill_fast_op(const OpPlan* p, FastOp<float>& a);
void fast_geometry(int axis, int n, const int* dims_in, long long* sa, long long* sb, long long* rs, int* na,
                   dim3* grid);

// Instantiated per operator kind in x3d_lines_<kind>.cu (FP32 only).
template <int KIND>
int fast_dispatch(const FastArgs<float>& a, bool xl, int L, dim3 grid, size_t smem, cudaStream_t st);

}  // namespace lk
}  // namespace x3d
