// Periodic spectral Poisson solve for sm_103a: src/poisson.f90:298-410
// (poisson_000) with the modified wavenumbers of waves (src/poisson.f90:
// 1530-1810).
//
// Five passes over the spectrum, each a batch of 1-D FFTs done entirely in
// shared memory (mixed radix 8/4/2 Stockham autosort, one radix-8 group of
// values per thread per pass):
//   A  x: real-to-complex (packed half-length complex FFT + split), nx/2+1 modes
//   B  y: forward complex FFT
//   C  z: forward FFT -> division by the modified wavenumber -> inverse FFT,
//      fused in one kernel so the z-spectrum never goes back to HBM between them
//   D  y: inverse complex FFT
//   E  x: complex-to-real
// The reference's half-cell shift factors (ax, bx, ...) are applied and then
// removed within poisson_000 itself; their product is exactly one, so the
// solve reduces to p_hat = -rhs_hat / (K * nx*ny*nz), with the reference's
// rule that modes with K < 1e-16 are set to zero.  K is evaluated with
// unfused IEEE multiplies and adds in the reference's order, so the zeroing
// decision is bit-identical to the reference's.
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "x3d_internal.h"

namespace x3d {

namespace {

constexpr int FFT_THREADS = 256;
constexpr int FFT_VALS = 8;  // complex values held per thread per pass
constexpr int FFT_ELEMS = FFT_THREADS * FFT_VALS;  // complex values per CTA

// Shared-memory line layout of the FFT kernels: element r of a line at
// r + r/8 (one pad slot per 8 elements), lines fft_ls(n) apart.  A Stockham
// pass writes 8 consecutive elements per thread; with the pad every store
// instruction of a warp touches each bank quad at most 4 times (the minimum
// for 16-byte elements) instead of 32.
__host__ __device__ __forceinline__ int fft_pad(int r) { return r + (r >> 3); }
__host__ __device__ __forceinline__ int fft_ls(int n) { return n + (n >> 3) + 1; }

// ---------------------------------------------------------------------------
// Arithmetic policies.  double / float: native complex arithmetic.  DF: every
// real number is an unevaluated sum hi + lo of two binary32 numbers (about a
// 48-bit significand), added with the error-free two-sum and multiplied with
// the FMA two-product, so FP64-class transforms run on GB300's FP32 pipes
// (its FP64 pipe is 1/64 of the FP32 rate).  A DF complex is 16 bytes, the
// size of a double2, so buffers and shared-memory tiles are unchanged.
// ---------------------------------------------------------------------------
struct DF {};
struct df { float h, l; };
struct __align__(16) cdf { float rh, rl, ih, il; };

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return df{s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df a, df b) {
  const df s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ df df_neg(df a) { return df{-a.h, -a.l}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
// Sum without the final renormalisation: hi is the rounded sum of the hi
// parts, lo collects their exact rounding error and the lo parts.  Used for
// the inner levels of a butterfly only (at most three in a row, the third
// feeding a product), whose last level renormalises: the error stays a few
// 2^-48 of the operands' size.
__device__ __forceinline__ df df_add_l(df a, df b) {
  const df s = two_sum(a.h, b.h);
  return df{s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l))};
}
__device__ __forceinline__ df df_sub_l(df a, df b) { return df_add_l(a, df_neg(b)); }
// x.h*y.h + u.h*v.h (sg = +1) or x.h*y.h - u.h*v.h (sg = -1) with the exact
// product errors and the cross terms folded into one lo sum, then one
// renormalisation: the real or imaginary part of a complex product in 19
// binary32 operations instead of 25, within a few 2^-48 of |a||b| (about
// 1.5x the error of separately renormalised products).
template <int SG>
__device__ __forceinline__ df df_dot2(df x, df y, df u, df v) {
  const float p1 = __fmul_rn(x.h, y.h);
  const float p2 = __fmul_rn(SG > 0 ? u.h : -u.h, v.h);
  const float e1 = __fmaf_rn(x.h, y.h, -p1);
  const float e2 = __fmaf_rn(SG > 0 ? u.h : -u.h, v.h, -p2);
  const df s = two_sum(p1, p2);
  float t = __fadd_rn(s.l, __fadd_rn(e1, e2));
  t = __fmaf_rn(x.h, y.l, t);
  t = __fmaf_rn(x.l, y.h, t);
  t = __fmaf_rn(SG > 0 ? u.h : -u.h, v.l, t);
  t = __fmaf_rn(SG > 0 ? u.l : -u.l, v.h, t);
  return fast_two_sum(s.h, t);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_half(df a) { return df{0.5f * a.h, 0.5f * a.l}; }  // exact
__device__ __forceinline__ df df_from(double d) {
  const float h = __double2float_rn(d);
  return df{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double df_to(df a) { return (double)a.h + (double)a.l; }
// 1/b with one Newton step in DF
__device__ __forceinline__ df df_rcp(df b) {
  const float r0 = 1.0f / b.h;
  const df br = df_mul(b, df{r0, 0.0f});
  const df e = df_sub(df{1.0f, 0.0f}, br);
  return df_add(df{r0, 0.0f}, df_mul(df{r0, 0.0f}, e));
}

template <typename R>
struct FT;

template <typename R>
struct FTnative {
  typedef typename std::conditional<std::is_same<R, double>::value, double2, float2>::type C;
  static __device__ __forceinline__ C add(C a, C b) { return C{a.x + b.x, a.y + b.y}; }
  static __device__ __forceinline__ C sub(C a, C b) { return C{a.x - b.x, a.y - b.y}; }
  static __device__ __forceinline__ C add_l(C a, C b) { return add(a, b); }
  static __device__ __forceinline__ C sub_l(C a, C b) { return sub(a, b); }
  static __device__ __forceinline__ C mul(C a, C b) { return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
  static __device__ __forceinline__ C conj(C a) { return C{a.x, -a.y}; }
  static __device__ __forceinline__ C half(C a) { return C{a.x * (R)0.5, a.y * (R)0.5}; }
  template <int S>
  static __device__ __forceinline__ C mul_i(C a) {  // a * (S*i)
    return S < 0 ? C{a.y, -a.x} : C{-a.y, a.x};
  }
  template <int S>
  static __device__ __forceinline__ C w8_1(C o) {
    const R h = (R)0.70710678118654752440084436210484903928;
    return S < 0 ? C{(o.x + o.y) * h, (o.y - o.x) * h} : C{(o.x - o.y) * h, (o.y + o.x) * h};
  }
  template <int S>
  static __device__ __forceinline__ C w8_3(C o) {
    const R h = (R)0.70710678118654752440084436210484903928;
    return S < 0 ? C{(o.y - o.x) * h, -(o.x + o.y) * h} : C{-(o.x + o.y) * h, (o.x - o.y) * h};
  }
  static __device__ __forceinline__ C from(double re, double im) { return C{(R)re, (R)im}; }
  static __device__ __forceinline__ C from_f(float re, float im) { return C{(R)re, (R)im}; }
  static __device__ __forceinline__ double re(C a) { return (double)a.x; }
  static __device__ __forceinline__ double im(C a) { return (double)a.y; }
  static __device__ __forceinline__ float re_f(C a) { return (float)a.x; }
  static __device__ __forceinline__ float im_f(C a) { return (float)a.y; }
  static __device__ __forceinline__ C zero() { return C{(R)0, (R)0}; }
};
template <>
struct FT<double> : FTnative<double> {};
template <>
struct FT<float> : FTnative<float> {};

template <>
struct FT<DF> {
  typedef cdf C;
  static __device__ __forceinline__ df R_(C a) { return df{a.rh, a.rl}; }
  static __device__ __forceinline__ df I_(C a) { return df{a.ih, a.il}; }
  static __device__ __forceinline__ C mk(df r, df i) { return C{r.h, r.l, i.h, i.l}; }
  static __device__ __forceinline__ C add(C a, C b) { return mk(df_add(R_(a), R_(b)), df_add(I_(a), I_(b))); }
  static __device__ __forceinline__ C sub(C a, C b) { return mk(df_sub(R_(a), R_(b)), df_sub(I_(a), I_(b))); }
  static __device__ __forceinline__ C add_l(C a, C b) { return mk(df_add_l(R_(a), R_(b)), df_add_l(I_(a), I_(b))); }
  static __device__ __forceinline__ C sub_l(C a, C b) { return mk(df_sub_l(R_(a), R_(b)), df_sub_l(I_(a), I_(b))); }
  static __device__ __forceinline__ C mul(C a, C b) {
    return mk(df_dot2<-1>(R_(a), R_(b), I_(a), I_(b)), df_dot2<1>(R_(a), I_(b), I_(a), R_(b)));
  }
  static __device__ __forceinline__ C conj(C a) { return C{a.rh, a.rl, -a.ih, -a.il}; }
  static __device__ __forceinline__ C half(C a) { return mk(df_half(R_(a)), df_half(I_(a))); }
  template <int S>
  static __device__ __forceinline__ C mul_i(C a) {
    return S < 0 ? C{a.ih, a.il, -a.rh, -a.rl} : C{-a.ih, -a.il, a.rh, a.rl};
  }
  static __device__ __forceinline__ df h_() { return df{0.70710677f, 1.2101617e-08f}; }  // 1/sqrt(2) as hi+lo
  template <int S>
  static __device__ __forceinline__ C w8_1(C o) {
    const df x = R_(o), y = I_(o), h = h_();
    return S < 0 ? mk(df_mul(df_add_l(x, y), h), df_mul(df_sub_l(y, x), h))
                 : mk(df_mul(df_sub_l(x, y), h), df_mul(df_add_l(y, x), h));
  }
  template <int S>
  static __device__ __forceinline__ C w8_3(C o) {
    const df x = R_(o), y = I_(o), h = h_();
    return S < 0 ? mk(df_mul(df_sub_l(y, x), h), df_neg(df_mul(df_add_l(x, y), h)))
                 : mk(df_neg(df_mul(df_add_l(x, y), h)), df_mul(df_sub_l(x, y), h));
  }
  static __device__ __forceinline__ C from(double re, double im) { return mk(df_from(re), df_from(im)); }
  // binary32 values are exact hi parts: no binary64 arithmetic on the way in
  static __device__ __forceinline__ C from_f(float re, float im) { return C{re, 0.f, im, 0.f}; }
  static __device__ __forceinline__ double re(C a) { return df_to(R_(a)); }
  static __device__ __forceinline__ double im(C a) { return df_to(I_(a)); }
  // nearest binary32 of hi + lo (|lo| <= ulp(hi) / 2: one rounding)
  static __device__ __forceinline__ float re_f(C a) { return __fadd_rn(a.rh, a.rl); }
  static __device__ __forceinline__ float im_f(C a) { return __fadd_rn(a.ih, a.il); }
  static __device__ __forceinline__ C zero() { return C{0.f, 0.f, 0.f, 0.f}; }
};

template <typename P>
struct Cx {
  typedef typename FT<P>::C T;
};

template <int SIGN, typename P, typename C>
__device__ __forceinline__ void fft2(C& a, C& b) {
  C t = a;
  a = FT<P>::add(t, b);
  b = FT<P>::sub(t, b);
}

// INNER: the outputs feed further butterfly levels (inside fft8) and are left
// unnormalised in double-float arithmetic; else the last level renormalises.
template <int SIGN, typename P, bool INNER = false, typename C>
__device__ __forceinline__ void fft4(C& x0, C& x1, C& x2, C& x3) {
  typedef FT<P> F;
  C s02 = F::add_l(x0, x2), d02 = F::sub_l(x0, x2);
  C s13 = F::add_l(x1, x3), d13 = F::template mul_i<SIGN>(F::sub_l(x1, x3));
  if (INNER) {
    x0 = F::add_l(s02, s13);
    x2 = F::sub_l(s02, s13);
    x1 = F::add_l(d02, d13);
    x3 = F::sub_l(d02, d13);
  } else {
    x0 = F::add(s02, s13);
    x2 = F::sub(s02, s13);
    x1 = F::add(d02, d13);
    x3 = F::sub(d02, d13);
  }
}

template <int SIGN, typename P, typename C>
__device__ __forceinline__ void fft8(C* v) {
  typedef FT<P> F;
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  fft4<SIGN, P, true>(e0, e1, e2, e3);
  fft4<SIGN, P, true>(o0, o1, o2, o3);
  C t1 = F::template w8_1<SIGN>(o1);
  C t2 = F::template mul_i<SIGN>(o2);
  C t3 = F::template w8_3<SIGN>(o3);
  v[0] = F::add(e0, o0); v[4] = F::sub(e0, o0);
  v[1] = F::add(e1, t1); v[5] = F::sub(e1, t1);
  v[2] = F::add(e2, t2); v[6] = F::sub(e2, t2);
  v[3] = F::add(e3, t3); v[7] = F::sub(e3, t3);
}

// One Stockham pass of radix R over `nl` lines of length n held in smem
// (line l at buf + l*lstride).  tw[m] = exp(SIGN*2*pi*i*m/n).  n, R and Ns
// are powers of two (ln = log2 n, lns = log2 Ns): index arithmetic by shifts
// and masks.
template <int R, int SIGN, typename P, typename C>
__device__ __forceinline__ void stockham_pass(C* buf, int lstride, int n, int ln, int nl, int Ns, int lns,
                                              const C* tw) {
  constexpr int G = FFT_VALS / R;  // butterflies per thread
  constexpr int LR = (R == 8) ? 3 : (R == 4) ? 2 : 1;
  const int lpl = ln - LR;  // log2(per_line)
  const int per_line = 1 << lpl;
  const int total = per_line * nl;
  const int lstep = ln - lns - LR;  // log2(n / (Ns R))
  C v[G][R];
  int base[G], off[G];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int bt = threadIdx.x + g * FFT_THREADS;
    base[g] = -1;
    if (bt < total) {
      const int l = bt >> lpl, j = bt & (per_line - 1);
      C* line = buf + l * lstride;
      const int kk = j & (Ns - 1);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        C x = line[fft_pad(j + r * per_line)];
        if (r > 0 && kk > 0) x = FT<P>::mul(x, tw[((kk * r) << lstep) & (n - 1)]);
        v[g][r] = x;
      }
      if (R == 8) fft8<SIGN, P>(v[g]);
      if (R == 4) fft4<SIGN, P>(v[g][0], v[g][1], v[g][2], v[g][3]);
      if (R == 2) fft2<SIGN, P>(v[g][0], v[g][1]);
      base[g] = l * lstride;
      off[g] = ((j >> lns) << (lns + LR)) + kk;
    }
  }
  __syncthreads();
#pragma unroll
  for (int g = 0; g < G; ++g)
    if (base[g] >= 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) buf[base[g] + fft_pad(off[g] + r * Ns)] = v[g][r];
    }
  __syncthreads();
}

template <int SIGN, typename P, typename C>
__device__ void smem_fft(C* buf, int lstride, int n, int nl, const C* tw) {
  // nl * n <= FFT_ELEMS: one radix group of FFT_VALS values per thread; n a
  // power of two
  const int ln = __ffs(n) - 1;
  int Ns = 1, lns = 0;
  int rem = n;
  while (rem >= 8) { stockham_pass<8, SIGN, P>(buf, lstride, n, ln, nl, Ns, lns, tw); Ns *= 8; lns += 3; rem >>= 3; }
  if (rem == 4) { stockham_pass<4, SIGN, P>(buf, lstride, n, ln, nl, Ns, lns, tw); Ns *= 4; lns += 2; rem >>= 2; }
  if (rem == 2) { stockham_pass<2, SIGN, P>(buf, lstride, n, ln, nl, Ns, lns, tw); }
}

// Lines per CTA of a strided pass: one radix group of values per thread
// (wider CTAs with fewer resident per SM measured slower at 512^3).
template <typename C>
int strided_lanes(int n) {
  return std::max(1, std::min(32, FFT_ELEMS / n));
}

// ---- Pass A: x real-to-complex --------------------------------------------
// Lines of nx reals -> nx/2+1 complex.  M = nx/2, packed z[m] = x[2m] + i x[2m+1].
template <typename P, typename TI = double>
__global__ void __launch_bounds__(FFT_THREADS, 4) fft_x_r2c(const TI* __restrict__ in,
                                                         typename Cx<P>::T* __restrict__ out, int nx, long long nlines,
                                                         int lpb, const typename Cx<P>::T* __restrict__ tw_half,
                                                         const typename Cx<P>::T* __restrict__ tw_full) {
  typedef typename Cx<P>::T C;
  typedef FT<P> F;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int M = nx / 2, nxh = M + 1;
  const long long l0 = (long long)blockIdx.x * lpb;
  const int nl = (int)min((long long)lpb, nlines - l0);
  const int lm = __ffs(M) - 1, ls = fft_ls(M);  // M a power of two
  if (std::is_same<TI, float>::value) {
    const float2* src = reinterpret_cast<const float2*>(in + l0 * nx);
    for (int e = threadIdx.x; e < nl * M; e += FFT_THREADS) {
      const float2 d = src[e];  // (x[2m], x[2m+1]) of line e / M
      buf[(e >> lm) * ls + fft_pad(e & (M - 1))] = F::from_f(d.x, d.y);
    }
  } else {
    const double2* src = reinterpret_cast<const double2*>(in + l0 * nx);
    for (int e = threadIdx.x; e < nl * M; e += FFT_THREADS) {
      const double2 d = src[e];
      buf[(e >> lm) * ls + fft_pad(e & (M - 1))] = F::from(d.x, d.y);
    }
  }
  __syncthreads();
  smem_fft<-1, P>(buf, ls, M, nl, tw_half);
  C* dst = out + l0 * nxh;
  // modes k = 0..M-1 by shift / mask, the k = M mode of each line after them
  for (int e = threadIdx.x; e < nl * (M + 1); e += FFT_THREADS) {
    const bool last = e >= nl * M;
    const int l = last ? e - nl * M : (e >> lm), k = last ? M : (e & (M - 1));
    const C* z = buf + l * ls;
    const C zk = z[fft_pad(k & (M - 1))], zn = F::conj(z[fft_pad((M - k) & (M - 1))]);
    // E = (Z[k] + conj Z[M-k])/2, O = (Z[k] - conj Z[M-k])/(2i), X = E + W^k O
    const C E = F::half(F::add(zk, zn));
    const C O = F::half(F::template mul_i<-1>(F::sub(zk, zn)));
    dst[(long long)l * nxh + k] = F::add(E, F::mul(tw_full[k], O));
  }
}

// ---- Pass E: x complex-to-real (unnormalised inverse) ----------------------
template <typename P, typename TO = double>
__global__ void __launch_bounds__(FFT_THREADS, 4) fft_x_c2r(const typename Cx<P>::T* __restrict__ in,
                                                         TO* __restrict__ out, int nx, long long nlines, int lpb,
                                                         const typename Cx<P>::T* __restrict__ tw_half_inv,
                                                         const typename Cx<P>::T* __restrict__ tw_full) {
  typedef typename Cx<P>::T C;
  typedef FT<P> F;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int M = nx / 2, nxh = M + 1;
  const long long l0 = (long long)blockIdx.x * lpb;
  const int nl = (int)min((long long)lpb, nlines - l0);
  const C* src = in + l0 * nxh;
  const int lm = __ffs(M) - 1, ls = fft_ls(M);  // M a power of two
  for (int e = threadIdx.x; e < nl * M; e += FFT_THREADS) {
    const int l = e >> lm, k = e & (M - 1);
    const C xk = src[(long long)l * nxh + k];
    const C xn = F::conj(src[(long long)l * nxh + (M - k)]);
    // E = X[k] + conj X[M-k]; O = (X[k] - conj X[M-k]) * conj(W^k); Z = E + i O
    const C E = F::add(xk, xn);
    const C O = F::mul(F::sub(xk, xn), F::conj(tw_full[k]));
    buf[l * ls + fft_pad(k)] = F::add(E, F::template mul_i<1>(O));
  }
  __syncthreads();
  smem_fft<1, P>(buf, ls, M, nl, tw_half_inv);
  if (std::is_same<TO, float>::value) {
    float2* dst = reinterpret_cast<float2*>(out + l0 * nx);
    for (int e = threadIdx.x; e < nl * M; e += FFT_THREADS) {
      const C z = buf[(e >> lm) * ls + fft_pad(e & (M - 1))];
      dst[e] = float2{F::re_f(z), F::im_f(z)};
    }
  } else {
    double2* dst = reinterpret_cast<double2*>(out + l0 * nx);
    for (int e = threadIdx.x; e < nl * M; e += FFT_THREADS) {
      const C z = buf[(e >> lm) * ls + fft_pad(e & (M - 1))];
      dst[e] = double2{F::re(z), F::im(z)};
    }
  }
}

// ---- Passes B/D (and C): strided complex FFTs -------------------------------
// Lines of length n with element stride `rs`; `lanes` consecutive lines
// (stride 1) per CTA, `nb` outer blocks with stride `bs`.
struct Spec {
  const double* k2[3];
  const double* tr[3];
  const float2* k2df[3];  // hi/lo split of k2 / tr (DF policy)
  const float2* trdf[3];
  int nx, ny, nz;
  double scale;  // 1/(nx*ny*nz)
  // optional per-mode factor -scale/K (0 where K < 1e-16), layout of the
  // spectrum, in the policy's number format (double, float, hi/lo float2)
  const void* inv;
};

// K of poisson_000's kxyz (src/poisson.f90:1688-1724, periodic): unfused IEEE
// binary64 in the reference's order, so the zeroing decision is the reference's.
__device__ __forceinline__ double kxyz64(const Spec& sp, int kx, int ky, int kz) {
  const double tx = sp.tr[0][kx], ty = sp.tr[1][ky], tz = sp.tr[2][kz];
  const double pyz = __dmul_rn(ty, tz), pxz = __dmul_rn(tx, tz), pxy = __dmul_rn(tx, ty);
  return __dadd_rn(__dadd_rn(__dmul_rn(sp.k2[0][kx], __dmul_rn(pyz, pyz)), __dmul_rn(sp.k2[1][ky], __dmul_rn(pxz, pxz))),
                   __dmul_rn(sp.k2[2][kz], __dmul_rn(pxy, pxy)));
}

template <typename P>
struct Spectral {
  // v / (-K nx ny nz), or 0 where K < 1e-16
  static __device__ __forceinline__ typename Cx<P>::T apply(typename Cx<P>::T v, const Spec& sp, int kx, int ky,
                                                            int kz) {
    typedef typename Cx<P>::T C;
    const double kk = kxyz64(sp, kx, ky, kz);
    if (kk < 1.0e-16) return FT<P>::zero();
    const double f = -sp.scale / kk;
    return C{(decltype(v.x))(v.x * f), (decltype(v.y))(v.y * f)};
  }
};

template <>
struct Spectral<DF> {
  static __device__ __forceinline__ cdf apply(cdf v, const Spec& sp, int kx, int ky, int kz) {
    const float2 tx2 = sp.trdf[0][kx], ty2 = sp.trdf[1][ky], tz2 = sp.trdf[2][kz];
    const float2 ax = sp.k2df[0][kx], ay = sp.k2df[1][ky], az = sp.k2df[2][kz];
    const df tx{tx2.x, tx2.y}, ty{ty2.x, ty2.y}, tz{tz2.x, tz2.y};
    const df pyz = df_mul(ty, tz), pxz = df_mul(tx, tz), pxy = df_mul(tx, ty);
    df kk = df_add(df_add(df_mul(df{ax.x, ax.y}, df_mul(pyz, pyz)), df_mul(df{ay.x, ay.y}, df_mul(pxz, pxz))),
                   df_mul(df{az.x, az.y}, df_mul(pxy, pxy)));
    if (kk.h < 1.0e-12f) {
      // near the zeroing threshold: decide and scale from the exact binary64 K
      const double k64 = kxyz64(sp, kx, ky, kz);
      if (k64 < 1.0e-16) return cdf{0.f, 0.f, 0.f, 0.f};
      kk = df_from(k64);
    }
    const df sc = df_from(-sp.scale);  // uniform; one conversion per mode
    const df f = df_mul(sc, df_rcp(kk));
    return FT<DF>::mk(df_mul(FT<DF>::R_(v), f), df_mul(FT<DF>::I_(v), f));
  }
};

// Multiply a mode by its tabulated factor.
template <typename P>
struct InvMul;
template <>
struct InvMul<double> {
  static __device__ __forceinline__ double2 mul(double2 v, const void* t, long long i) {
    const double f = reinterpret_cast<const double*>(t)[i];
    return make_double2(v.x * f, v.y * f);
  }
};
template <>
struct InvMul<float> {
  static __device__ __forceinline__ float2 mul(float2 v, const void* t, long long i) {
    const float f = reinterpret_cast<const float*>(t)[i];
    return make_float2(v.x * f, v.y * f);
  }
};
template <>
struct InvMul<DF> {
  static __device__ __forceinline__ cdf mul(cdf v, const void* t, long long i) {
    const float2 f2 = reinterpret_cast<const float2*>(t)[i];
    const df f{f2.x, f2.y};
    return FT<DF>::mk(df_mul(FT<DF>::R_(v), f), df_mul(FT<DF>::I_(v), f));
  }
};

// Per-mode factor table -scale/K of poisson_000 (K and the zeroing rule as in
// kxyz64), built once per context and number format.
template <typename P>
__global__ void k_inv_table(void* out, Spec sp) {
  const int nxh = sp.nx / 2 + 1;
  const long long n = (long long)nxh * sp.ny * sp.nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % nxh);
    const int ky = (int)((i / nxh) % sp.ny);
    const int kz = (int)(i / ((long long)nxh * sp.ny));
    const double kk = kxyz64(sp, kx, ky, kz);
    const double f = (kk < 1.0e-16) ? 0.0 : -sp.scale / kk;
    if (std::is_same<P, double>::value) {
      reinterpret_cast<double*>(out)[i] = f;
    } else if (std::is_same<P, float>::value) {
      reinterpret_cast<float*>(out)[i] = (float)f;
    } else {
      const float h = (float)f;
      reinterpret_cast<float2*>(out)[i] = make_float2(h, (float)(f - (double)h));
    }
  }
}

template <typename P, bool POISSON, int SIGN>
__global__ void __launch_bounds__(FFT_THREADS, 4) fft_strided(typename Cx<P>::T* __restrict__ data, int n, long long rs,
                                                           int na, int lanes, long long bs,
                                                           const typename Cx<P>::T* __restrict__ tw_f,
                                                           const typename Cx<P>::T* __restrict__ tw_i, Spec sp) {
  typedef typename Cx<P>::T C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int lstride = fft_ls(n);
  const int a0 = blockIdx.x * lanes;
  const int nl = min(lanes, na - a0);
  const long long b = blockIdx.y;
  C* base = data + b * bs + a0;
  const int llan = __ffs(lanes) - 1, lnn = __ffs(n) - 1;  // lanes, n: powers of two
  for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
    const int r = e >> llan, l = e & (lanes - 1);
    if (l < nl) buf[l * lstride + fft_pad(r)] = base[r * rs + l];
  }
  __syncthreads();
  smem_fft<SIGN, P>(buf, lstride, n, nl, SIGN < 0 ? tw_f : tw_i);
  if (POISSON) {
    // z-lines: a = kx (0..nx/2), b = ky; row r = kz
    if (sp.inv) {
      const int nxh = sp.nx / 2 + 1;
      for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
        const int l = e >> lnn, kz = e & (n - 1);
        const long long i = ((long long)kz * sp.ny + b) * nxh + a0 + l;
        buf[l * lstride + fft_pad(kz)] = InvMul<P>::mul(buf[l * lstride + fft_pad(kz)], sp.inv, i);
      }
    } else {
      for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
        const int l = e >> lnn, kz = e & (n - 1);
        buf[l * lstride + fft_pad(kz)] = Spectral<P>::apply(buf[l * lstride + fft_pad(kz)], sp, a0 + l, (int)b, kz);
      }
    }
    __syncthreads();
    smem_fft<1, P>(buf, lstride, n, nl, tw_i);
  }
  for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
    const int r = e >> llan, l = e & (lanes - 1);
    if (l < nl) base[r * rs + l] = buf[l * lstride + fft_pad(r)];
  }
}

bool pow2(int n) { return n >= 2 && (n & (n - 1)) == 0; }

}  // namespace

// Twiddle storage layout in the context (double and float copies):
//   [0, nx/2)            forward  exp(-2 pi i m/(nx/2))
//   [.., +nx/2)          inverse
//   [.., +nx/2+1)        exp(-2 pi i k/nx), k = 0..nx/2   (x split)
//   [.., +ny)            forward ny, then inverse ny
//   [.., +nz)            forward nz, then inverse nz
static void twiddles(int n, int sign, std::vector<double>& out) {
  const long double twopi = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < n; ++m) {
    const long double ang = sign * twopi * (long double)m / (long double)n;
    out.push_back((double)cosl(ang));
    out.push_back((double)sinl(ang));
  }
}

static int fft_setup(Ctx* c) {
  if (c->d_twid) return X3D_OK;
  const int nx = c->grid.nx, ny = c->grid.ny, nz = c->grid.nz;
  std::vector<double> t;
  twiddles(nx / 2, -1, t);
  twiddles(nx / 2, +1, t);
  {
    const long double twopi = 6.283185307179586476925286766559005768L;
    for (int k = 0; k <= nx / 2; ++k) {
      const long double ang = -twopi * (long double)k / (long double)nx;
      t.push_back((double)cosl(ang));
      t.push_back((double)sinl(ang));
    }
  }
  twiddles(ny, -1, t);
  twiddles(ny, +1, t);
  twiddles(nz, -1, t);
  twiddles(nz, +1, t);
  std::vector<float> t32(t.size()), tdf(2 * t.size());
  for (size_t i = 0; i < t.size(); ++i) {
    t32[i] = (float)t[i];
    tdf[2 * i] = (float)t[i];
    tdf[2 * i + 1] = (float)(t[i] - (double)tdf[2 * i]);
  }
  if (cudaMalloc(&c->d_twid, t.size() * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
  if (cudaMalloc(&c->d_twid32, t32.size() * sizeof(float)) != cudaSuccess) return X3D_ERR_NOMEM;
  if (cudaMalloc(&c->d_twid_df, tdf.size() * sizeof(float)) != cudaSuccess) return X3D_ERR_NOMEM;
  cudaMemcpy(c->d_twid, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_twid32, t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_twid_df, tdf.data(), tdf.size() * sizeof(float), cudaMemcpyHostToDevice);
  c->twid_n = (int)t.size() / 2;
  // Poisson tables (binary64 and hi/lo binary32 pairs)
  for (int ax = 0; ax < 3; ++ax) {
    dvec k2, tr;
    waves_tables(c->ax[ax], k2, tr);
    std::vector<float> k2s(2 * k2.size()), trs(2 * tr.size());
    for (size_t i = 0; i < k2.size(); ++i) {
      k2s[2 * i] = (float)k2[i];
      k2s[2 * i + 1] = (float)(k2[i] - (double)k2s[2 * i]);
      trs[2 * i] = (float)tr[i];
      trs[2 * i + 1] = (float)(tr[i] - (double)trs[2 * i]);
    }
    if (cudaMalloc(&c->d_k2[ax], k2.size() * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
    if (cudaMalloc(&c->d_tr[ax], tr.size() * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
    if (cudaMalloc(&c->d_k2df[ax], k2s.size() * sizeof(float)) != cudaSuccess) return X3D_ERR_NOMEM;
    if (cudaMalloc(&c->d_trdf[ax], trs.size() * sizeof(float)) != cudaSuccess) return X3D_ERR_NOMEM;
    cudaMemcpy(c->d_k2[ax], k2.data(), k2.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_tr[ax], tr.data(), tr.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_k2df[ax], k2s.data(), k2s.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_trdf[ax], trs.data(), trs.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  return cuda_status(cudaGetLastError());
}

template <typename R, typename TIO = double>
static int poisson_run(Ctx* c, TIO* rhs, cudaStream_t st) {
  typedef typename Cx<R>::T C;
  const int nx = c->grid.nx, ny = c->grid.ny, nz = c->grid.nz;
  const int M = nx / 2, nxh = M + 1;
  const size_t need = (size_t)nxh * ny * nz * sizeof(C);
  if (c->fft_work_bytes < need) {
    if (c->fft_work) cudaFree(c->fft_work);
    c->fft_work = nullptr;
    c->fft_work_bytes = 0;
    if (cudaMalloc(&c->fft_work, need) != cudaSuccess) return X3D_ERR_NOMEM;
    c->fft_work_bytes = need;
  }
  C* spec = reinterpret_cast<C*>(c->fft_work);
  const void* twv = std::is_same<R, double>::value ? (const void*)c->d_twid
                    : std::is_same<R, float>::value ? (const void*)c->d_twid32
                                                    : (const void*)c->d_twid_df;
  const C* tw = reinterpret_cast<const C*>(twv);
  const C* twx_f = tw;
  const C* twx_i = tw + M;
  const C* twx_full = tw + 2 * M;
  const C* twy_f = twx_full + nxh;
  const C* twy_i = twy_f + ny;
  const C* twz_f = twy_i + ny;
  const C* twz_i = twz_f + nz;

  Spec sp;
  for (int a = 0; a < 3; ++a) {
    sp.k2[a] = c->d_k2[a];
    sp.tr[a] = c->d_tr[a];
    sp.k2df[a] = c->d_k2df[a];
    sp.trdf[a] = c->d_trdf[a];
  }
  sp.nx = nx; sp.ny = ny; sp.nz = nz;
  sp.scale = 1.0 / ((double)nx * (double)ny * (double)nz);
  sp.inv = nullptr;
  {
    // per-mode factor table, built on first use for this number format
    const int slot = std::is_same<R, double>::value ? 0 : std::is_same<R, float>::value ? 1 : 2;
    if (!c->d_inv[slot]) {
      const size_t es = slot == 1 ? sizeof(float) : sizeof(double);
      void* t = nullptr;
      if (cudaMalloc(&t, (size_t)nxh * ny * nz * es) != cudaSuccess) return X3D_ERR_NOMEM;
      k_inv_table<R><<<4 * c->num_sms, 256, 0, st>>>(t, sp);
      c->d_inv[slot] = t;
    }
    sp.inv = c->d_inv[slot];
  }

  // A: x r2c
  {
    const long long nlines = (long long)ny * nz;
    const int lpb = std::max(1, FFT_ELEMS / std::max(M, 1));
    const size_t smem = (size_t)lpb * fft_ls(M) * sizeof(C);
    auto k = fft_x_r2c<R, TIO>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const unsigned nb = (unsigned)((nlines + lpb - 1) / lpb);
    k<<<nb, FFT_THREADS, smem, st>>>(rhs, spec, nx, nlines, lpb, twx_f, twx_full);
  }
  // B: y forward, lines over kx with stride nxh, outer over z
  const int lanes_y = strided_lanes<C>(ny);
  const size_t smem_y = (size_t)lanes_y * fft_ls(ny) * sizeof(C);
  {
    auto k = fft_strided<R, false, -1>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_y);
    dim3 g((nxh + lanes_y - 1) / lanes_y, nz);
    k<<<g, FFT_THREADS, smem_y, st>>>(spec, ny, nxh, nxh, lanes_y, (long long)nxh * ny, twy_f, twy_i, sp);
  }
  // C: z forward + Poisson + z inverse; lines over kx, outer over ky
  {
    const int lanes_z = strided_lanes<C>(nz);
    const size_t smem_z = (size_t)lanes_z * fft_ls(nz) * sizeof(C);
    auto k = fft_strided<R, true, -1>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_z);
    dim3 g((nxh + lanes_z - 1) / lanes_z, ny);
    k<<<g, FFT_THREADS, smem_z, st>>>(spec, nz, (long long)nxh * ny, nxh, lanes_z, nxh, twz_f, twz_i, sp);
  }
  // D: y inverse
  {
    auto k = fft_strided<R, false, 1>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_y);
    dim3 g((nxh + lanes_y - 1) / lanes_y, nz);
    k<<<g, FFT_THREADS, smem_y, st>>>(spec, ny, nxh, nxh, lanes_y, (long long)nxh * ny, twy_f, twy_i, sp);
  }
  // E: x c2r
  {
    const long long nlines = (long long)ny * nz;
    const int lpb = std::max(1, FFT_ELEMS / std::max(M, 1));
    const size_t smem = (size_t)lpb * fft_ls(M) * sizeof(C);
    auto k = fft_x_c2r<R, TIO>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const unsigned nb = (unsigned)((nlines + lpb - 1) / lpb);
    k<<<nb, FFT_THREADS, smem, st>>>(spec, rhs, nx, nlines, lpb, twx_i, twx_full);
  }
  return cuda_status(cudaGetLastError());
}

static int periodic_shape_ok(const Ctx* c) {
  const int nx = c->grid.nx, ny = c->grid.ny, nz = c->grid.nz;
  if (!c->ax[0].periodic || !c->ax[1].periodic || !c->ax[2].periodic) return X3D_ERR_BC;
  if (!pow2(nx) || !pow2(ny) || !pow2(nz) || nx < 16 || ny < 8 || nz < 8) return X3D_ERR_UNSUPPORTED;
  if (nx / 2 > FFT_ELEMS || ny > FFT_ELEMS / 1 || nz > FFT_ELEMS) return X3D_ERR_UNSUPPORTED;
  if ((long long)ny * nz > (1LL << 31) || ny > 65535 || nz > 65535) return X3D_ERR_UNSUPPORTED;
  return X3D_OK;
}

int poisson_periodic_f32io(Ctx* c, float* p, cudaStream_t st) {
  int rc = periodic_shape_ok(c);
  if (rc == X3D_OK) rc = fft_setup(c);
  if (rc != X3D_OK) return rc;
  return poisson_run<DF, float>(c, p, st);
}

int poisson_periodic(Ctx* c, double* rhs, int precision, cudaStream_t st) {
  const int nx = c->grid.nx, ny = c->grid.ny, nz = c->grid.nz;
  if (!c->ax[0].periodic || !c->ax[1].periodic || !c->ax[2].periodic) return X3D_ERR_BC;
  if (!pow2(nx) || !pow2(ny) || !pow2(nz) || nx < 16 || ny < 8 || nz < 8) return X3D_ERR_UNSUPPORTED;
  if (nx / 2 > FFT_ELEMS || ny > FFT_ELEMS / 1 || nz > FFT_ELEMS) return X3D_ERR_UNSUPPORTED;
  if ((long long)ny * nz > (1LL << 31) || ny > 65535 || nz > 65535) return X3D_ERR_UNSUPPORTED;
  int rc = fft_setup(c);
  if (rc != X3D_OK) return rc;
  if (precision == 0) return poisson_run<double>(c, rhs, st);
  if (precision == 1) return poisson_run<float>(c, rhs, st);
  if (precision == 2) return poisson_run<DF>(c, rhs, st);
  return X3D_ERR_DTYPE;
}

// ---------------------------------------------------------------------------
// Allocation-free Poisson solve (x3d_poisson_noalloc).
//
// Some callers cannot allocate device memory at the point where they solve:
// codes that reserve the whole device up front in their own memory pool (a
// caching allocator, or a solver that sizes every buffer at start-up and
// treats a later allocation as an error), or that call from a context where a
// cudaMalloc would be refused.  This variant takes its spectrum and its
// twiddle / wavenumber tables from one fixed array in device memory instead
// of the context's lazily allocated buffers, and calls no allocating routine.
//
// The array below is part of the library's device image: every GPU that
// loads the library holds these 64 MiB until the process exits.  All calls
// (from any context, on any stream) share it and it keeps the previous call's
// contents; each call rewrites the tables and the whole spectrum before
// reading them, so nothing needs clearing, but two calls that overlap on the
// GPU race on it.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocBytes = size_t(X3D_NOALLOC_SCRATCH_BYTES);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {nullptr};

// Device address of the scratch array for the current device.  Host code may
// not use the symbol's name as an address; the address is fetched once per
// device (with that device current) and cached.  The first call on a device
// does this set-up, so it should come before any stream capture.
int noalloc_scratch(int dev, unsigned char** out) {
  if (dev < 0 || dev >= 64) return X3D_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e);
    g_noalloc_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_addr[dev]);
  return X3D_OK;
}

struct WaveAxis {
  int n;
  double len, d, aci6, bci6, alcai6, aici6, bici6, cici6, dici6, ailcai6;
};

WaveAxis wave_axis(const AxisCoef& a) {
  return WaveAxis{a.n, a.len, a.d, a.aci6, a.bci6, a.alcai6, a.aici6, a.bici6, a.cici6s, a.dici6, a.ailcai6};
}

__device__ void tw_entry(double2* t, int m, int n, double sign) {
  double s, c;
  sincospi(2.0 * (double)m / (double)n, &s, &c);
  *t = double2{c, sign * s};
}

// Twiddles (same layout as the context's table) and the modified-wavenumber /
// transfer tables of the periodic waves() branch, written into the scratch.
__global__ void k_noalloc_tables(double2* tw, double* k2, double* tr, int nx, int ny, int nz, WaveAxis ax,
                                 WaveAxis ay, WaveAxis az) {
  const int M = nx / 2;
  const int ntw = 3 * M + 1 + 2 * ny + 2 * nz;
  const double twopi = 6.283185307179586476925286766559;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ntw + nx + ny + nz; q += gridDim.x * blockDim.x) {
    if (q < ntw) {
      int m = q;
      if (m < M) { tw_entry(tw + q, m, M, -1.0); continue; }
      m -= M;
      if (m < M) { tw_entry(tw + q, m, M, 1.0); continue; }
      m -= M;
      if (m <= M) { tw_entry(tw + q, m, nx, -1.0); continue; }
      m -= M + 1;
      if (m < ny) { tw_entry(tw + q, m, ny, -1.0); continue; }
      m -= ny;
      if (m < ny) { tw_entry(tw + q, m, ny, 1.0); continue; }
      m -= ny;
      if (m < nz) { tw_entry(tw + q, m, nz, -1.0); continue; }
      m -= nz;
      tw_entry(tw + q, m, nz, 1.0);
      continue;
    }
    int i = q - ntw;
    const WaveAxis* a = &ax;
    int off = 0;
    if (i >= nx) { i -= nx; off += nx; a = &ay; if (i >= ny) { i -= ny; off += ny; a = &az; } }
    const int n = a->n;
    const int ii = (i <= n / 2) ? i : n - i;  // tables are symmetric in the mode index
    const double w = twopi * ii / n;
    double wp = a->aci6 * 2.0 * a->d * sin(w * 0.5) + a->bci6 * 2.0 * a->d * sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * a->alcai6 * cos(w));
    const double kk = n * wp / a->len;
    k2[off + i] = kk * kk;
    const double rl = (n * w / a->len) * a->d;
    const double tt = 2.0 * (a->bici6 * cos(rl * 1.5) + a->cici6 * cos(rl * 2.5) + a->dici6 * cos(rl * 3.5));
    const double tt1 = 2.0 * a->aici6 * cos(rl * 0.5);
    const double t1 = 1.0 + 2.0 * a->ailcai6 * cos(rl);
    tr[off + i] = (tt1 + tt) / t1;
  }
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

int poisson_periodic_noalloc(Ctx* c, double* rhs, cudaStream_t st) {
  typedef double2 C;
  const int nx = c->grid.nx, ny = c->grid.ny, nz = c->grid.nz;
  if (!c->ax[0].periodic || !c->ax[1].periodic || !c->ax[2].periodic) return X3D_ERR_BC;
  if (!pow2(nx) || !pow2(ny) || !pow2(nz) || nx < 16 || ny < 8 || nz < 8) return X3D_ERR_UNSUPPORTED;
  if (nx / 2 > FFT_ELEMS || ny > FFT_ELEMS || nz > FFT_ELEMS) return X3D_ERR_UNSUPPORTED;
  const int M = nx / 2, nxh = M + 1;
  const size_t ntw = (size_t)3 * M + 1 + 2 * ny + 2 * nz;
  const size_t b_tw = align256(ntw * sizeof(C));
  const size_t b_tab = align256((size_t)(nx + ny + nz) * sizeof(double));
  const size_t b_spec = (size_t)nxh * ny * nz * sizeof(C);
  if (b_tw + 2 * b_tab + b_spec > kNoAllocBytes) return X3D_ERR_SCRATCH;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev != c->device) return X3D_ERR_ARG;
  unsigned char* base = nullptr;
  int rc = noalloc_scratch(dev, &base);
  if (rc != X3D_OK) return rc;
  C* tw = reinterpret_cast<C*>(base);
  double* k2 = reinterpret_cast<double*>(base + b_tw);
  double* tr = reinterpret_cast<double*>(base + b_tw + b_tab);
  C* spec = reinterpret_cast<C*>(base + b_tw + 2 * b_tab);
  k_noalloc_tables<<<64, 256, 0, st>>>(tw, k2, tr, nx, ny, nz, wave_axis(c->ax[0]), wave_axis(c->ax[1]),
                                       wave_axis(c->ax[2]));
  rc = cuda_status(cudaGetLastError());
  if (rc != X3D_OK) return rc;
  const C* twx_f = tw;
  const C* twx_i = tw + M;
  const C* twx_full = tw + 2 * M;
  const C* twy_f = twx_full + nxh;
  const C* twy_i = twy_f + ny;
  const C* twz_f = twy_i + ny;
  const C* twz_i = twz_f + nz;
  Spec sp;
  std::memset(&sp, 0, sizeof(sp));
  sp.k2[0] = k2; sp.k2[1] = k2 + nx; sp.k2[2] = k2 + nx + ny;
  sp.tr[0] = tr; sp.tr[1] = tr + nx; sp.tr[2] = tr + nx + ny;
  sp.nx = nx; sp.ny = ny; sp.nz = nz;
  sp.scale = 1.0 / ((double)nx * (double)ny * (double)nz);
  const long long nlines = (long long)ny * nz;
  const int lpb = std::max(1, FFT_ELEMS / std::max(M, 1));
  const size_t smem_x = (size_t)lpb * fft_ls(M) * sizeof(C);
  const unsigned nbx = (unsigned)((nlines + lpb - 1) / lpb);
  const int lanes_y = std::max(1, std::min(32, FFT_ELEMS / ny));
  const size_t smem_y = (size_t)lanes_y * fft_ls(ny) * sizeof(C);
  const int lanes_z = std::max(1, std::min(32, FFT_ELEMS / nz));
  const size_t smem_z = (size_t)lanes_z * fft_ls(nz) * sizeof(C);
  auto kr2c = fft_x_r2c<double>;
  auto kyf = fft_strided<double, false, -1>;
  auto kz = fft_strided<double, true, -1>;
  auto kyi = fft_strided<double, false, 1>;
  auto kc2r = fft_x_c2r<double>;
  if ((e = cudaFuncSetAttribute(kr2c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(kyf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_y)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(kz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_z)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(kyi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_y)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(kc2r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x)) != cudaSuccess)
    return cuda_status(e);
  kr2c<<<nbx, FFT_THREADS, smem_x, st>>>(rhs, spec, nx, nlines, lpb, twx_f, twx_full);
  kyf<<<dim3((nxh + lanes_y - 1) / lanes_y, nz), FFT_THREADS, smem_y, st>>>(spec, ny, nxh, nxh, lanes_y,
                                                                           (long long)nxh * ny, twy_f, twy_i, sp);
  kz<<<dim3((nxh + lanes_z - 1) / lanes_z, ny), FFT_THREADS, smem_z, st>>>(spec, nz, (long long)nxh * ny, nxh,
                                                                          lanes_z, nxh, twz_f, twz_i, sp);
  kyi<<<dim3((nxh + lanes_y - 1) / lanes_y, nz), FFT_THREADS, smem_y, st>>>(spec, ny, nxh, nxh, lanes_y,
                                                                           (long long)nxh * ny, twy_f, twy_i, sp);
  kc2r<<<nbx, FFT_THREADS, smem_x, st>>>(spec, rhs, nx, nlines, lpb, twx_i, twx_full);
  return cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// poisson_010: x and z periodic, y non-periodic (src/poisson.f90:665-1013).
//
// The reference reorders y (even points forward, odd points backward), takes
// a 3-D FFT, turns the y-spectrum into a cosine spectrum with the half-sample
// combination of modes j and ny-j (src/poisson.f90:764-785), solves in y
// (division by kxyz, or on a stretched mesh the two pentadiagonal systems of
// the odd and even modes, src/poisson.f90:834-880 with src/tools.f90:
// 1225-1362) and undoes everything.  The x and z half-cell shift factors
// cancel as in poisson_000, and the y reorder commutes with the x and z
// transforms, so the GPU does:
//   A  x real-to-complex;  B  z forward FFT;
//   C  one kernel per batch of (kx, kz) lines: gather y in reordered order,
//      forward FFT, cosine combination, solve, inverse combination, inverse
//      FFT, scatter back in reordered order -- the y-spectrum stays in shared
//      memory;
//   D  z inverse FFT;  E  x complex-to-real.
// The pentadiagonal coefficients are formed on the fly per line from 1-D
// tables (matrice_refinement's formulas), one thread per (line, odd/even
// system), and eliminated in the reference's order with its epsilon guards.
// ---------------------------------------------------------------------------
namespace {

struct P010 {
  const double *kx2, *trx, *kz2, *trz;  // x (nx/2+1 used) and z (nz, mirrored) tables
  const double *yk2, *ty, *yky, *say, *sby;  // y tables, nym entries
  const double2 *twy_f, *twy_i;
  double xa0, xa1, scale;
  int istret, nx, nz, nym, nsolve;  // nsolve = threads of the solve phase (2 per line)
};

__device__ __forceinline__ double2 cosine_fwd(double2 v, double2 w, double ay, double by) {
  const double x1 = v.x * by, x2 = v.x * ay, x3 = v.y * by, x4 = v.y * ay;
  const double x5 = w.x * by, x6 = w.x * ay, x7 = w.y * by, x8 = w.y * ay;
  return make_double2(0.5 * (x1 + x4 + x5 - x8), 0.5 * (-x2 + x3 + x6 + x7));
}
__device__ __forceinline__ double2 cosine_bwd(double2 v, double2 w, double ay, double by) {
  const double x1 = v.x * by, x2 = v.x * ay, x3 = v.y * by, x4 = v.y * ay;
  const double x5 = w.x * by, x6 = w.x * ay, x7 = w.y * by, x8 = w.y * ay;
  return make_double2(x1 - x4 + x6 + x7, -(-x2 - x3 + x5 - x8));
}

// Pentadiagonal solve of one (kx, kz) line's odd (sys 0) or even (sys 1) y
// modes, in place on e[2m + sys], m = 0..nh-1.  band: 5 diagonals x nh rows,
// interleaved over the T solve threads (entry (q, m) at band[(q*nh + m)*T]).
__device__ void penta_line(double2* e, double* band, int T, int nh, int sys, int kx, int kz, const P010& q) {
  auto B = [&](int qq, int m) -> double& { return band[(size_t)(qq * nh + m) * T]; };
  const double kx2 = q.kx2[kx], kz2 = q.kz2[kz], tx = q.trx[kx], tz = q.trz[kz];
  const double tx2 = tx * tx, tz2 = tz * tz;
  const double xa0 = q.xa0, xa1 = q.xa1;
  const double xa0_2 = xa0 * xa0, xa1_2 = xa1 * xa1, xa01 = xa0 * xa1, xa0p1_2 = (xa0 + xa1) * (xa0 + xa1);
  auto cw = [&](int m) { return tx * (q.yky[2 * m + sys] * tz); };
  auto ty2 = [&](int m) { const double t = q.ty[2 * m + sys]; return t * t; };
  // diagonals (matrice_refinement, src/poisson.f90:1925-2113)
  for (int m = 0; m < nh; ++m) {
    const double c0 = cw(m);
    const double cm = m > 0 ? cw(m - 1) : 0.0, cp = m + 1 < nh ? cw(m + 1) : 0.0;
    double a2c = xa0_2, nb = cm + cp;
    if (m == 0) { nb = cp; if (sys == 1) a2c = xa0_2 - xa1_2; }
    if (m == nh - 1) { nb = cm; if (sys == 1) a2c = xa0p1_2; }
    B(2, m) = -(kx2 * ty2(m) * tz2 + kz2 * ty2(m) * tx2 + a2c * (c0 * c0) + xa1_2 * c0 * nb);
    B(3, m) = (m + 1 < nh) ? xa01 * (cp * (c0 + cp)) : 0.0;
    B(4, m) = (m + 2 < nh) ? xa1_2 * (-(cp * cw(m + 2))) : 0.0;
    B(1, m) = (m > 0) ? xa01 * (cm * (c0 + cm)) : 0.0;
    B(0, m) = (m > 1) ? xa1_2 * (-(cm * cw(m - 2))) : 0.0;
  }
  {
    const double c0 = cw(0), c1 = cw(1);
    if (sys == 0) {
      B(3, 0) = 2.0 * xa01 * (c0 * c1 + c1 * c1);
      B(4, 0) = 2.0 * B(4, 0);
    } else {
      B(3, 0) = (xa0 - xa1) * xa1 * (c0 * c1) + xa0 * xa1 * (c1 * c1);
      B(1, 1) = xa0 * xa1 * (c1 * c0) + (xa0 + xa1) * xa1 * (c0 * c0);
      const double ca = cw(nh - 2), cb = cw(nh - 1);
      B(3, nh - 2) = xa0 * xa1 * ca * cb + (xa0 + xa1) * xa1 * (cb * cb);
      B(1, nh - 1) = (xa0 + xa1) * xa1 * (cb * ca) + xa0 * xa1 * (ca * ca);
    }
    B(4, nh - 2) = 0.0;
    if (sys == 0 && kx2 == 0.0 && kz2 == 0.0) {
      B(2, 0) = 1.0; B(3, 0) = 0.0; B(4, 0) = 0.0;
    }
  }
  // inversion5_v1: forward elimination
  const double eps = 1.0e-16;
  auto E = [&](int m) -> double2& { return e[fft_pad(2 * m + sys)]; };
  double tmp = 0.0;
  for (int m = 0; m <= nh - 3; ++m)
    for (int ii = 1; ii <= 2; ++ii) {
      const int mi = m + ii;
      const double piv = B(2, m);
      if (piv != 0.0) tmp = B(2 - ii, mi) / piv;
      const double2 em = E(m), emi = E(mi);
      E(mi) = make_double2(emi.x - tmp * em.x, emi.y - tmp * em.y);
      const int j0 = (ii == 1) ? 2 : 1;
      for (int jc = j0; jc <= j0 + 1; ++jc) B(jc, mi) = B(jc, mi) - tmp * B(jc + ii, m);
    }
  {
    const double p1 = B(2, nh - 2);
    const double sr = (fabs(p1) > eps) ? B(1, nh - 1) / p1 : 0.0;
    const double b1 = B(2, nh - 1) - sr * B(3, nh - 2);
    const double2 en = E(nh - 1), en1 = E(nh - 2);
    double2 t3 = make_double2(0.0, 0.0);
    if (fabs(b1) > eps) {
      const double t1 = sr / b1;
      t3 = make_double2(en.x / b1 - t1 * en1.x, en.y / b1 - t1 * en1.y);
    }
    E(nh - 1) = t3;
    const double r = (fabs(p1) > eps) ? 1.0 / p1 : 0.0;
    const double a1 = B(3, nh - 2) * r;
    E(nh - 2) = make_double2(en1.x * r - a1 * t3.x, en1.y * r - a1 * t3.y);
  }
  for (int i = nh - 3; i >= 0; --i) {
    const double p = B(2, i);
    const double r = (fabs(p) > eps) ? 1.0 / p : 0.0;
    const double a1 = B(3, i) * r, b1 = B(4, i) * r;
    const double2 e0 = E(i), e1 = E(i + 1), e2 = E(i + 2);
    E(i) = make_double2(e0.x * r - a1 * e1.x - b1 * e2.x, e0.y * r - a1 * e1.y - b1 * e2.y);
  }
}

// Pass C.  Lines: kx = blockIdx.x*lanes + l (stride 1), kz = blockIdx.y; the
// y row stride is rs = nx/2+1, the kz plane stride bs = (nx/2+1)*nym.
__global__ void __launch_bounds__(FFT_THREADS, 4) k_p010_y(double2* __restrict__ data, long long rs, int na, int lanes,
                                                        long long bs, P010 q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = q.nym, nh = n / 2, ls = fft_ls(n);
  double2* buf = reinterpret_cast<double2*>(smem_raw);
  double* band = reinterpret_cast<double*>(buf + (size_t)lanes * ls);
  const int a0 = blockIdx.x * lanes;
  const int nl = min(lanes, na - a0);
  const int kz = blockIdx.y;
  double2* base = data + (long long)kz * bs + a0;
  // gather in the reordered y order (src/poisson.f90:688-698)
  for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
    const int r = e / lanes, l = e - r * lanes;
    const int src = (r < nh) ? 2 * r : 2 * n - 2 * r - 1;
    if (l < nl) buf[l * ls + fft_pad(r)] = base[src * rs + l];
  }
  __syncthreads();
  smem_fft<-1, double>(buf, ls, n, nl, q.twy_f);
  // cosine combination of modes j and n-j, with the 1/(nx nym nz) normalisation
  for (int e = threadIdx.x; e < nl * nh; e += FFT_THREADS) {
    const int l = e / nh, j = 1 + (e - l * nh), jp = n - j;
    double2* line = buf + l * ls;
    const double2 v = line[fft_pad(j)], w = line[fft_pad(jp)];
    const double2 sv = make_double2(v.x * q.scale, v.y * q.scale), sw = make_double2(w.x * q.scale, w.y * q.scale);
    line[fft_pad(j)] = cosine_fwd(sv, sw, q.say[j], q.sby[j]);
    if (jp != j) line[fft_pad(jp)] = cosine_fwd(sw, sv, q.say[jp], q.sby[jp]);
    if (j == 1) line[0] = make_double2(line[0].x * q.scale, line[0].y * q.scale);
  }
  __syncthreads();
  if (q.istret == 0) {
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, j = e - l * n;
      const int kx = a0 + l;
      const double pyz = __dmul_rn(q.ty[j], q.trz[kz]), pxz = __dmul_rn(q.trx[kx], q.trz[kz]),
                   pxy = __dmul_rn(q.trx[kx], q.ty[j]);
      const double kk = __dadd_rn(__dadd_rn(__dmul_rn(q.kx2[kx], __dmul_rn(pyz, pyz)), __dmul_rn(q.yk2[j], __dmul_rn(pxz, pxz))),
                                  __dmul_rn(q.kz2[kz], __dmul_rn(pxy, pxy)));
      double2& v = buf[l * ls + fft_pad(j)];
      if (fabs(kk) < 1.0e-16) v = make_double2(0.0, 0.0);
      else v = make_double2(v.x / (-kk), v.y / (-kk));
    }
  } else if (threadIdx.x < 2 * nl) {
    const int l = threadIdx.x >> 1, sys = threadIdx.x & 1;
    penta_line(buf + l * ls, band + threadIdx.x, q.nsolve, nh, sys, a0 + l, kz, q);
  }
  __syncthreads();
  // the (nx/2, nz/2) line is zeroed (src/poisson.f90:887-894)
  if (kz == q.nz / 2)
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, j = e - l * n;
      if (a0 + l == q.nx / 2) buf[l * ls + fft_pad(j)] = make_double2(0.0, 0.0);
    }
  __syncthreads();
  for (int e = threadIdx.x; e < nl * nh; e += FFT_THREADS) {
    const int l = e / nh, j = 1 + (e - l * nh), jp = n - j;
    double2* line = buf + l * ls;
    const double2 v = line[fft_pad(j)], w = line[fft_pad(jp)];
    line[fft_pad(j)] = cosine_bwd(v, w, q.say[j], q.sby[j]);
    if (jp != j) line[fft_pad(jp)] = cosine_bwd(w, v, q.say[jp], q.sby[jp]);
  }
  __syncthreads();
  smem_fft<1, double>(buf, ls, n, nl, q.twy_i);
  for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
    const int r = e / lanes, l = e - r * lanes;
    const int dst = (r < nh) ? 2 * r : 2 * n - 2 * r - 1;
    if (l < nl) base[dst * rs + l] = buf[l * ls + fft_pad(r)];
  }
}

}  // namespace

// Device tables of poisson_010 (one block of doubles):
//   yk2 | ty | yky | say | sby (nym each) | twy_f | twy_i (2*nym each);
// the stretching constants xa0, xa1 stay on the host (kernel arguments).
static int p010_setup(Ctx* c) {
  if (c->d_p010) return X3D_OK;
  const AxisCoef& ay = c->ax[1];
  const int nym = ay.nm;
  dvec yky, yk2, tr, sa, sb;
  waves_y010(ay, c->st.istret, c->grid.yly, yky, yk2, tr, sa, sb);
  dvec h;
  h.insert(h.end(), yk2.begin(), yk2.begin() + nym);
  h.insert(h.end(), tr.begin(), tr.end());
  h.insert(h.end(), yky.begin(), yky.begin() + nym);
  h.insert(h.end(), sa.begin(), sa.end());
  h.insert(h.end(), sb.begin(), sb.end());
  std::vector<double> tw;
  twiddles(nym, -1, tw);
  twiddles(nym, +1, tw);
  h.insert(h.end(), tw.begin(), tw.end());
  const double pi = std::acos(-1.0), alpha = c->st.alpha, beta = c->st.beta;
  double xa0 = 0, xa1 = 0;
  if (c->st.istret == 1 || c->st.istret == 2) {
    xa0 = alpha / pi + 0.5 / beta / pi;
    xa1 = (c->st.istret == 1) ? 1.0 / 4.0 / beta / pi : -(1.0 / 4.0 / beta / pi);
  }
  c->p010_xa[0] = xa0;
  c->p010_xa[1] = xa1;
  double* d = nullptr;
  if (cudaMalloc(&d, h.size() * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
  cudaError_t e = cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_status(e);
  }
  c->d_p010 = d;
  return X3D_OK;
}

int poisson_010(Ctx* c, double* rhs, cudaStream_t st) {
  const int nx = c->grid.nx, nz = c->grid.nz, nym = c->ax[1].nm;
  if (!c->ax[0].periodic || c->ax[1].periodic || !c->ax[2].periodic) return X3D_ERR_BC;
  if (c->st.istret == 3) return X3D_ERR_UNSUPPORTED;  // inversion5_v2 path
  if (!pow2(nx) || !pow2(nz) || !pow2(nym) || nx < 16 || nz < 8 || nym < 8) return X3D_ERR_UNSUPPORTED;
  if (nx / 2 > FFT_ELEMS || nz > FFT_ELEMS || nym > 1024 || nz > 65535) return X3D_ERR_UNSUPPORTED;
  int rc = fft_setup(c);
  if (rc == X3D_OK) rc = p010_setup(c);
  if (rc != X3D_OK) return rc;
  typedef double2 C;
  const int M = nx / 2, nxh = M + 1, ny = c->grid.ny;
  const size_t need = (size_t)nxh * nym * nz * sizeof(C);
  if (c->fft_work_bytes < need) {
    if (c->fft_work) cudaFree(c->fft_work);
    c->fft_work = nullptr;
    c->fft_work_bytes = 0;
    if (cudaMalloc(&c->fft_work, need) != cudaSuccess) return X3D_ERR_NOMEM;
    c->fft_work_bytes = need;
  }
  C* spec = reinterpret_cast<C*>(c->fft_work);
  const C* tw = reinterpret_cast<const C*>(c->d_twid);
  const C* twx_f = tw;
  const C* twx_i = tw + M;
  const C* twx_full = tw + 2 * M;
  const C* twz_f = twx_full + nxh + 2 * ny;
  const C* twz_i = twz_f + nz;
  P010 q;
  const double* t = c->d_p010;
  q.kx2 = c->d_k2[0]; q.trx = c->d_tr[0]; q.kz2 = c->d_k2[2]; q.trz = c->d_tr[2];
  q.yk2 = t; q.ty = t + nym; q.yky = t + 2 * nym; q.say = t + 3 * nym; q.sby = t + 4 * nym;
  q.twy_f = reinterpret_cast<const double2*>(t + 5 * nym);
  q.twy_i = q.twy_f + nym;
  q.istret = c->st.istret;
  q.nx = nx; q.nz = nz; q.nym = nym;
  q.scale = 1.0 / ((double)nx * (double)nym * (double)nz);
  q.xa0 = c->p010_xa[0];
  q.xa1 = c->p010_xa[1];
  Spec sp{};
  // A: x r2c
  const long long nlines = (long long)nym * nz;
  const int lpb = std::max(1, FFT_ELEMS / std::max(M, 1));
  const size_t smem_x = (size_t)lpb * fft_ls(M) * sizeof(C);
  const unsigned nbx = (unsigned)((nlines + lpb - 1) / lpb);
  {
    auto k = fft_x_r2c<double>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x);
    k<<<nbx, FFT_THREADS, smem_x, st>>>(rhs, spec, nx, nlines, lpb, twx_f, twx_full);
  }
  // B: z forward; lines over kx, outer over y
  const int lanes_z = strided_lanes<C>(nz);
  const size_t smem_z = (size_t)lanes_z * fft_ls(nz) * sizeof(C);
  const dim3 gz((nxh + lanes_z - 1) / lanes_z, nym);
  {
    auto k = fft_strided<double, false, -1>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_z);
    k<<<gz, FFT_THREADS, smem_z, st>>>(spec, nz, (long long)nxh * nym, nxh, lanes_z, nxh, twz_f, twz_i, sp);
  }
  // C: y reorder + cosine transform + solve
  {
    const int nh = nym / 2;
    int lanes = std::max(1, std::min(16, FFT_ELEMS / nym));
    auto smem_of = [&](int ln) { return (size_t)ln * fft_ls(nym) * sizeof(C) + (size_t)(2 * ln) * 5 * nh * sizeof(double); };
    while (lanes > 1 && smem_of(lanes) > 200 * 1024) lanes /= 2;
    const size_t smem = smem_of(lanes);
    q.nsolve = 2 * lanes;
    cudaFuncSetAttribute(k_p010_y, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const dim3 g((nxh + lanes - 1) / lanes, nz);
    k_p010_y<<<g, FFT_THREADS, smem, st>>>(spec, nxh, nxh, lanes, (long long)nxh * nym, q);
  }
  // D: z inverse
  {
    auto k = fft_strided<double, false, 1>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_z);
    k<<<gz, FFT_THREADS, smem_z, st>>>(spec, nz, (long long)nxh * nym, nxh, lanes_z, nxh, twz_f, twz_i, sp);
  }
  // E: x c2r
  {
    auto k = fft_x_c2r<double>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x);
    k<<<nbx, FFT_THREADS, smem_x, st>>>(spec, rhs, nx, nlines, lpb, twx_i, twx_full);
  }
  return cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// poisson_11x (src/poisson.f90:1019-1465): x and y free-slip, z free-slip
// (bcz = 1) or periodic (bcz = 0), uniform mesh, FP64.  p-mesh NX x NY x NZ
// (nxm, nym, nzm), spectrum NX x NY x (NZ/2+1) as 2DECOMP's PHYSICAL_IN_Z
// transform leaves it.  The reference transforms the reordered field in 3-D,
// then post-processes mode pairs (k, n-k) axis by axis, divides by kxyz, and
// undoes the steps in reverse.  Each post-processing is a complex-linear map
// along its own axis (a e + b conj(e)) / 2, so it commutes with the other
// axes' transforms; here each axis is one kernel: gather (even / odd
// reorder) + FFT + its post-processing, the x kernel also scales, divides
// and runs the backward x steps, and the last kernel does the z
// complex-to-real transform and the inverse reorder.
// ---------------------------------------------------------------------------
namespace {

struct P11 {
  int NX, NY, NZ, NZ2, bcz;
  const double2 *twx_f, *twx_i, *twy_f, *twy_i, *twz_f, *twz_i;
  const double *sax, *sbx, *say, *sby, *saz, *sbz;
  const double2* kxyz;
};

__device__ __forceinline__ int slip_perm(int d, int n) { return (d < n / 2) ? 2 * d : 2 * n - 2 * d - 1; }

// forward mode-pair combination of src/poisson.f90:1138-1156, written as there
__device__ __forceinline__ double2 p11_fwd(double2 a, double2 b, double bb, double aa) {
  const double x1 = a.x * bb * 0.5, x2 = a.x * aa * 0.5, x3 = a.y * bb * 0.5, x4 = a.y * aa * 0.5;
  const double x5 = b.x * bb * 0.5, x6 = b.x * aa * 0.5, x7 = b.y * bb * 0.5, x8 = b.y * aa * 0.5;
  return make_double2(x1 + x4 + x5 - x8, -x2 + x3 + x6 + x7);
}
// backward combination of src/poisson.f90:1340-1356
__device__ __forceinline__ double2 p11_bwd(double2 a, double2 b, double bb, double aa) {
  const double x1 = a.x * bb, x2 = a.x * aa, x3 = a.y * bb, x4 = a.y * aa;
  const double x5 = b.x * bb, x6 = b.x * aa, x7 = b.y * bb, x8 = b.y * aa;
  return make_double2(x1 - x4 + x6 + x7, -(-x2 - x3 + x5 - x8));
}

enum { P11_ZF = 0, P11_YF = 1, P11_X = 2, P11_YB = 3, P11_ZB = 4 };

// One kernel per stage; a block holds `lanes` lines of length n in shared
// memory (buf) plus a second buffer for the mode-pair combination.
template <int MODE>
__global__ void __launch_bounds__(FFT_THREADS, 4) k_p11(double2* __restrict__ W, double* __restrict__ rhs, P11 q,
                                                     int lanes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = (MODE == P11_X) ? q.NX : (MODE == P11_YF || MODE == P11_YB) ? q.NY : q.NZ;
  const int ls = fft_ls(n);
  double2* buf = reinterpret_cast<double2*>(smem_raw);
  double2* bf2 = buf + (size_t)lanes * ls;
  const int NX = q.NX, NY = q.NY, NZ = q.NZ, NZ2 = q.NZ2;
  const int a0 = blockIdx.x * lanes, b = blockIdx.y;
  const int na = (MODE == P11_X) ? NY : NX;
  const int nl = min(lanes, na - a0);
  // spectral index of (line l, row r); lines are consecutive i (y, z stages)
  // or consecutive j (x stage)
  auto sidx = [&](int l, int r) -> size_t {
    if (MODE == P11_X) return (size_t)r + (size_t)NX * ((size_t)(a0 + l) + (size_t)NY * b);
    if (MODE == P11_YF || MODE == P11_YB) return (size_t)(a0 + l) + (size_t)NX * ((size_t)r + (size_t)NY * b);
    return (size_t)(a0 + l) + (size_t)NX * ((size_t)b + (size_t)NY * r);
  };
  // ---- load
  if (MODE == P11_ZF) {
    const int j = b, pj = slip_perm(j, NY);
    for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
      const int r = e / lanes, l = e - r * lanes;
      if (l < nl) {
        const int i = a0 + l, k = r;
        const int pk = q.bcz ? slip_perm(k, NZ) : k;
        buf[l * ls + fft_pad(r)] = make_double2(rhs[(size_t)slip_perm(i, NX) + (size_t)NX * ((size_t)pj + (size_t)NY * pk)], 0.0);
      }
    }
  } else if (MODE == P11_ZB) {
    for (int e = threadIdx.x; e < lanes * NZ2; e += FFT_THREADS) {
      const int r = e / lanes, l = e - r * lanes;
      if (l < nl) {
        const double2 v = W[sidx(l, r)];
        // backward z combination (src/poisson.f90:1395-1404)
        buf[l * ls + fft_pad(r)] = make_double2(v.x * q.sbz[r] - v.y * q.saz[r], v.y * q.sbz[r] + v.x * q.saz[r]);
      }
    }
    __syncthreads();
    // Hermitian extension: complex-to-real along z
    for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
      const int l = e / n, r = e - l * n;
      if (l < nl) {
        if (r >= NZ2) {
          const double2 v = buf[l * ls + fft_pad((n - r))];
          buf[l * ls + fft_pad(r)] = make_double2(v.x, -v.y);
        }
      }
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nl; l += FFT_THREADS) {
      buf[l * ls].y = 0.0;
      if ((n & 1) == 0) buf[l * ls + fft_pad(n / 2)].y = 0.0;
    }
  } else {
    for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
      int l, r;
      if (MODE == P11_X) { l = e / n; r = e - l * n; } else { r = e / lanes; l = e - r * lanes; }
      if (l < nl) buf[l * ls + fft_pad(r)] = W[sidx(l, r)];
    }
  }
  __syncthreads();
  // ---- pre-combination of the backward stages (x is done below)
  if (MODE == P11_YB) {
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, m = e - l * n;
      bf2[l * ls + fft_pad(m)] = (m == 0) ? buf[l * ls] : p11_bwd(buf[l * ls + fft_pad(m)], buf[l * ls + fft_pad(n - m)], q.sby[m], q.say[m]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, m = e - l * n;
      buf[l * ls + fft_pad(m)] = bf2[l * ls + fft_pad(m)];
    }
    __syncthreads();
  }
  // ---- transform
  const double2 *twf = (MODE == P11_X) ? q.twx_f : (MODE == P11_YF || MODE == P11_YB) ? q.twy_f : q.twz_f;
  const double2 *twi = (MODE == P11_X) ? q.twx_i : (MODE == P11_YF || MODE == P11_YB) ? q.twy_i : q.twz_i;
  if (MODE == P11_ZF || MODE == P11_YF || MODE == P11_X) smem_fft<-1, double>(buf, ls, n, nl, twf);
  else smem_fft<1, double>(buf, ls, n, nl, twi);
  // ---- post-combination of the forward stages
  if (MODE == P11_ZF) {
    for (int e = threadIdx.x; e < nl * NZ2; e += FFT_THREADS) {
      const int l = e / NZ2, k = e - l * NZ2;
      const double2 v = buf[l * ls + fft_pad(k)];
      // src/poisson.f90:1117-1126
      buf[l * ls + fft_pad(k)] = make_double2(v.x * q.sbz[k] + v.y * q.saz[k], v.y * q.sbz[k] - v.x * q.saz[k]);
    }
    __syncthreads();
  }
  if (MODE == P11_YF) {
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, m = e - l * n;
      bf2[l * ls + fft_pad(m)] = (m == 0) ? buf[l * ls] : p11_fwd(buf[l * ls + fft_pad(m)], buf[l * ls + fft_pad(n - m)], q.sby[m], q.say[m]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, m = e - l * n;
      buf[l * ls + fft_pad(m)] = bf2[l * ls + fft_pad(m)];
    }
    __syncthreads();
  }
  if (MODE == P11_X) {
    const int k = b;
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, m = e - l * n;
      double2 v = (m == 0) ? buf[l * ls] : p11_fwd(buf[l * ls + fft_pad(m)], buf[l * ls + fft_pad(n - m)], q.sbx[m], q.sax[m]);
      // normalisation (src/poisson.f90:1113-1114)
      v = make_double2(v.x / (double)NX / (double)NY / (double)NZ, v.y / (double)NX / (double)NY / (double)NZ);
      // division with the reference's guards (src/poisson.f90:1200-1224)
      const double2 kk = q.kxyz[(size_t)m + (size_t)NX * ((size_t)(a0 + l) + (size_t)NY * k)];
      const double eps = 1.0e-16;
      const bool r0 = fabs(kk.x) < eps, i0 = fabs(kk.y) < eps;
      if (r0 && i0) v = make_double2(0.0, 0.0);
      else if (r0) v = make_double2(0.0, v.y / (-kk.y));
      else if (i0) v = make_double2(v.x / (-kk.x), 0.0);
      else v = make_double2(v.x / (-kk.x), v.y / (-kk.y));
      bf2[l * ls + fft_pad(m)] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nl * n; e += FFT_THREADS) {
      const int l = e / n, m = e - l * n;
      buf[l * ls + fft_pad(m)] = (m == 0) ? bf2[l * ls] : p11_bwd(bf2[l * ls + fft_pad(m)], bf2[l * ls + fft_pad(n - m)], q.sbx[m], q.sax[m]);
    }
    __syncthreads();
    smem_fft<1, double>(buf, ls, n, nl, q.twx_i);
  }
  // ---- store
  if (MODE == P11_ZB) {
    const int j = b, pj = slip_perm(j, NY);
    for (int e = threadIdx.x; e < lanes * n; e += FFT_THREADS) {
      const int r = e / lanes, l = e - r * lanes;
      if (l < nl) {
        const int i = a0 + l, k = r;
        const int pk = q.bcz ? slip_perm(k, NZ) : k;
        rhs[(size_t)slip_perm(i, NX) + (size_t)NX * ((size_t)pj + (size_t)NY * pk)] = buf[l * ls + fft_pad(r)].x;
      }
    }
  } else {
    const int rows = (MODE == P11_ZF) ? NZ2 : n;
    for (int e = threadIdx.x; e < lanes * rows; e += FFT_THREADS) {
      int l, r;
      if (MODE == P11_X) { l = e / rows; r = e - l * rows; } else { r = e / lanes; l = e - r * lanes; }
      if (l < nl) W[sidx(l, r)] = buf[l * ls + fft_pad(r)];
    }
  }
}

}  // namespace

bool is_11x(const Ctx* c) {
  auto slip = [](const AxisCoef& a) { return a.ncl1 == 1 && a.ncln == 1; };
  return slip(c->ax[0]) && slip(c->ax[1]) && (c->ax[2].periodic || slip(c->ax[2]));
}

// Device tables of poisson_11x (one block of doubles):
//   twx_f | twx_i (2 NX each) | twy_f | twy_i | twz_f | twz_i | sax | sbx (NX)
//   | say | sby (NY) | saz | sbz (NZ) | kxyz (2 NX NY (NZ/2+1))
static int p11_setup(Ctx* c) {
  if (c->d_p11) return X3D_OK;
  const AxisCoef &ax = c->ax[0], &ay = c->ax[1], &az = c->ax[2];
  const int NX = ax.nm, NY = ay.nm, NZ = az.nm;
  const double pi = std::acos(-1.0);
  dvec h;
  twiddles(NX, -1, h);
  twiddles(NX, +1, h);
  twiddles(NY, -1, h);
  twiddles(NY, +1, h);
  twiddles(NZ, -1, h);
  twiddles(NZ, +1, h);
  // abxyz (src/poisson.f90:1469-1526): half-cell factors of free-slip axes,
  // the periodic factors for a periodic z
  auto ab = [&](int n, bool slip) {
    dvec a(n), bb(n);
    for (int i = 1; i <= n; ++i) {
      const double arg = slip ? (double)(i - 1) * pi * 0.5 / (double)n : (double)(i - 1) * pi / (double)n;
      a[i - 1] = std::sin(arg);
      bb[i - 1] = std::cos(arg);
    }
    h.insert(h.end(), a.begin(), a.end());
    h.insert(h.end(), bb.begin(), bb.end());
  };
  ab(NX, true);
  ab(NY, true);
  ab(NZ, !az.periodic);
  dvec kre, kim;
  kxyz_11x(ax, ay, az, kre, kim);
  for (size_t i = 0; i < kre.size(); ++i) {
    h.push_back(kre[i]);
    h.push_back(kim[i]);
  }
  double* d = nullptr;
  if (cudaMalloc(&d, h.size() * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
  cudaError_t e = cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_status(e);
  }
  c->d_p11 = d;
  return X3D_OK;
}

int poisson_11x(Ctx* c, double* rhs, cudaStream_t st) {
  if (!is_11x(c)) return X3D_ERR_BC;
  if (c->st.istret != 0) return X3D_ERR_UNSUPPORTED;  // matrice_refinement path of poisson_11x
  const int NX = c->ax[0].nm, NY = c->ax[1].nm, NZ = c->ax[2].nm, NZ2 = NZ / 2 + 1;
  if (!pow2(NX) || !pow2(NY) || !pow2(NZ) || NX < 8 || NY < 8 || NZ < 8) return X3D_ERR_UNSUPPORTED;
  if (NX > FFT_ELEMS || NY > FFT_ELEMS || NZ > FFT_ELEMS || NY > 65535 || NZ2 > 65535) return X3D_ERR_UNSUPPORTED;
  int rc = p11_setup(c);
  if (rc != X3D_OK) return rc;
  const size_t need = (size_t)NX * NY * NZ2 * sizeof(double2);
  if (c->fft_work_bytes < need) {
    if (c->fft_work) cudaFree(c->fft_work);
    c->fft_work = nullptr;
    c->fft_work_bytes = 0;
    if (cudaMalloc(&c->fft_work, need) != cudaSuccess) return X3D_ERR_NOMEM;
    c->fft_work_bytes = need;
  }
  double2* W = reinterpret_cast<double2*>(c->fft_work);
  P11 q;
  q.NX = NX; q.NY = NY; q.NZ = NZ; q.NZ2 = NZ2; q.bcz = c->ax[2].periodic ? 0 : 1;
  const double* t = c->d_p11;
  const double2* tw = reinterpret_cast<const double2*>(t);
  q.twx_f = tw; q.twx_i = tw + NX;
  q.twy_f = tw + 2 * NX; q.twy_i = q.twy_f + NY;
  q.twz_f = q.twy_i + NY; q.twz_i = q.twz_f + NZ;
  const double* s = t + 2 * (2 * NX + 2 * NY + 2 * NZ);
  q.sax = s; q.sbx = s + NX; s += 2 * NX;
  q.say = s; q.sby = s + NY; s += 2 * NY;
  q.saz = s; q.sbz = s + NZ; s += 2 * NZ;
  q.kxyz = reinterpret_cast<const double2*>(s);
  auto launch = [&](auto kern, int n, int na, int nb) -> int {
    const int lanes = std::max(1, std::min(32, FFT_ELEMS / n));
    const size_t smem = (size_t)2 * lanes * fft_ls(n) * sizeof(double2);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    const dim3 g((unsigned)((na + lanes - 1) / lanes), (unsigned)nb);
    kern<<<g, FFT_THREADS, smem, st>>>(W, rhs, q, lanes);
    return cuda_status(cudaGetLastError());
  };
  rc = launch(k_p11<P11_ZF>, NZ, NX, NY);
  if (rc == X3D_OK) rc = launch(k_p11<P11_YF>, NY, NX, NZ2);
  if (rc == X3D_OK) rc = launch(k_p11<P11_X>, NX, NY, NZ2);
  if (rc == X3D_OK) rc = launch(k_p11<P11_YB>, NY, NX, NZ2);
  if (rc == X3D_OK) rc = launch(k_p11<P11_ZB>, NZ, NX, NY);
  return rc;
}

}  // namespace x3d
