// Fused momentum right-hand side along one axis (FP32 fast path).
//
// For one velocity component u_q and one direction j the reference forms, with
// transposes between the stages (src/transeq.f90:73-591),
//   conv_j = d_j(u_j u_q) + u_j d_j u_q,      visc_j = d_jj u_q,
// and sums them into the right-hand side.  Here one kernel runs the three
// compact solves of a line (first derivative of the product, first derivative
// and second derivative of u_q) back to back on the same CTA:
//   out = nu * C(u_q) + a1 - (A(u_j u_q) + u_j B(u_q)) / 2
// so u_j, u_q and the running sum a1 are read from HBM once and out is written
// once (4 field passes instead of 11 with one kernel per solve).  The partial
// sum between solves stays in shared memory; re-reads of u_q / u_j for the
// later solves' windows hit L1/L2.  The arithmetic and its order are those of
// the unfused sequence (conv = A + u_j B; out = (nu C + a1) + (-1/2) conv).
#include "x3d_line_fast.cuh"

namespace x3d {
namespace lk {

struct RhsArgs {
  const float *ua, *uq, *a1;
  float* out;
  long long sa, sb, rs;
  int n, na;
  FastOp<float> A, B, C;  // d(ua uq), d(uq), dd(uq)
  float nu;
};

template <bool XL, int L>
__global__ void __launch_bounds__(LANES* FCHUNKS, 2) rhs_fast(const __grid_constant__ RhsArgs p) {
  constexpr int W1 = L + 4;  // first-derivative window (halo 2)
  constexpr int W2 = L + 8;  // second-derivative window (halo 4)
  constexpr int NT = LANES * FCHUNKS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* cfw = reinterpret_cast<float*>(smem_raw);
  float* cbw = cfw + FCHUNKS * LANES;
  float* ends = cbw + FCHUNKS * LANES;
  float* work = ends + 2 * LANES;

  const int lane = threadIdx.x, ch = threadIdx.y, tid = ch * LANES + lane;
  const int n = p.n;
  const int a0 = blockIdx.x * LANES;
  const long long b = blockIdx.y;
  const int nl = min(LANES, p.na - a0);
  const int r0 = ch * L;
  const bool edge = (ch == 0 || ch == FCHUNKS - 1);
  float v[L];

  if (!XL) {
    // y / z lines: windows straight from global memory; partial sums in smem
    float* stash = work;  // [L][NT]
    const bool ok = lane < nl;
    const long long off = (ok ? (long long)(a0 + lane) * p.sa : 0) + b * p.sb;
    const float* q = p.uq + off;
    const float* ua = p.ua + off;
    {
      float w[W1];
      load_window<float, W1>(w, q, ua, r0 - 2, n, p.rs, edge);
      fast_solve<float, K_DER1, L>(w, v, p.A, cfw, cbw, ends, ch, lane);
    }
#pragma unroll
    for (int k = 0; k < L; ++k) stash[k * NT + tid] = v[k];
    {
      float w[W1];
      load_window<float, W1>(w, q, nullptr, r0 - 2, n, p.rs, edge);
      fast_solve<float, K_DER1, L>(w, v, p.B, cfw, cbw, ends, ch, lane);
    }
    {
      const float* ub = ua + (long long)r0 * p.rs;
      const int s32 = (int)p.rs;
#pragma unroll
      for (int k = 0; k < L; ++k) {
        const float uj = ub[k * s32];
        stash[k * NT + tid] = stash[k * NT + tid] + uj * v[k];
      }
    }
    {
      float w[W2];
      load_window<float, W2>(w, q, nullptr, r0 - 4, n, p.rs, edge);
      fast_solve<float, K_DER2, L>(w, v, p.C, cfw, cbw, ends, ch, lane);
    }
    if (ok) {
      float* dst = p.out + off;
      const float* a1 = p.a1 ? p.a1 + off : nullptr;
      // a1 may alias out: each group of rows is read before it is written
      constexpr int G = 4;
#pragma unroll
      for (int k0 = 0; k0 < L; k0 += G) {
        float A1[G];
#pragma unroll
        for (int g = 0; g < G; ++g) A1[g] = a1 ? a1[(long long)(r0 + k0 + g) * p.rs] : 0.f;
#pragma unroll
        for (int g = 0; g < G; ++g) {
          float o = p.nu * v[k0 + g];
          if (a1) o = o + A1[g];
          o = o + (-0.5f) * stash[(k0 + g) * NT + tid];
          dst[(long long)(r0 + k0 + g) * p.rs] = o;
        }
      }
    }
  } else {
    // x lines: the 32 lines are transposed once into two tiles (u_q and the
    // product); the product tile then holds the partial sums
    float* tq = work;               // [n][LD]
    float* tp = work + n * LD;      // [n][LD], then the partial sums [L][NT]
    const long long off = (long long)a0 * p.sa + b * p.sb;
    for (int l = ch; l < LANES; l += FCHUNKS)
      for (int r = lane; r < n; r += LANES) {
        float qv = 0.f, av = 0.f;
        if (l < nl) {
          const long long i = off + (long long)l * p.sa + r;
          qv = p.uq[i];
          av = p.ua[i];
        }
        tq[r * LD + l] = qv;
        tp[r * LD + l] = qv * av;
      }
    __syncthreads();
    {
      float w[W1];
#pragma unroll
      for (int j = 0; j < W1; ++j) w[j] = tp[wrow(r0 - 2 + j, n, edge) * LD + lane];
      fast_solve<float, K_DER1, L>(w, v, p.A, cfw, cbw, ends, ch, lane);
    }
    // every thread read its product window before the solve's first barrier
    float* stash = tp;
#pragma unroll
    for (int k = 0; k < L; ++k) stash[k * NT + tid] = v[k];
    {
      float w[W1];
#pragma unroll
      for (int j = 0; j < W1; ++j) w[j] = tq[wrow(r0 - 2 + j, n, edge) * LD + lane];
      fast_solve<float, K_DER1, L>(w, v, p.B, cfw, cbw, ends, ch, lane);
    }
    const bool ok = lane < nl;
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const float uj = ok ? p.ua[off + (long long)lane * p.sa + r0 + k] : 0.f;
      stash[k * NT + tid] = stash[k * NT + tid] + uj * v[k];
    }
    {
      float w[W2];
#pragma unroll
      for (int j = 0; j < W2; ++j) w[j] = tq[wrow(r0 - 4 + j, n, edge) * LD + lane];
      fast_solve<float, K_DER2, L>(w, v, p.C, cfw, cbw, ends, ch, lane);
    }
    // the u_q tile is free (windows were read before the solve's barriers)
#pragma unroll
    for (int k = 0; k < L; ++k) tq[(r0 + k) * LD + lane] = v[k];
    __syncthreads();
    for (int l = ch; l < nl; l += FCHUNKS)
      for (int r = lane; r < n; r += LANES) {
        const long long i = off + (long long)l * p.sa + r;
        float o = p.nu * tq[r * LD + l];
        if (p.a1) o = o + p.a1[i];
        o = o + (-0.5f) * stash[(r % L) * NT + (r / L) * LANES + l];
        p.out[i] = o;
      }
  }
}

// ---- x lines: one warp per line -------------------------------------------
// For x lines the line is contiguous in memory, so a warp can own one line:
// the line is read (and the result written) coalesced through a padded
// per-warp buffer, lane t holds rows t*L .. t*L+L-1 (n = 32 L) in registers,
// and the chunk carries are combined with a warp-shuffle scan of the affine
// maps c_out = pf_end * c_in + y_end (Kogge-Stone, 5 steps): no block barrier.
constexpr int XCH = 32;  // chunks per line = lanes

struct WarpOp {
  const float *s, *f, *w, *pf, *qb, *rsm;
  float ca, cb, cc, cd, alpha, den;
  float s_inf, f_inf, w_inf, g_inf;
  float pfe[XCH], qbs[XCH];
  int mode[XCH];
  int nterms_int;
};

struct RhsXArgs {
  const float *ua, *uq, *a1;
  float* out;
  long long sa, sb;  // line and plane strides (row stride 1)
  int n, na;
  WarpOp A, B, C;
  float nu;
};

// Inclusive scan of affine maps x -> a x + b over the lanes (lane order
// forward when DOWN is false, backward when true); returns the carry into
// this lane (exclusive result).
template <bool DOWN>
__device__ __forceinline__ float carry_scan(float a, float b, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const float pa = DOWN ? __shfl_down_sync(0xffffffffu, a, d) : __shfl_up_sync(0xffffffffu, a, d);
    const float pb = DOWN ? __shfl_down_sync(0xffffffffu, b, d) : __shfl_up_sync(0xffffffffu, b, d);
    const bool in = DOWN ? (lane + d < 32) : (lane >= d);
    if (in) {
      b = a * pb + b;
      a = a * pa;
    }
  }
  const float e = DOWN ? __shfl_down_sync(0xffffffffu, b, 1) : __shfl_up_sync(0xffffffffu, b, 1);
  return (DOWN ? lane == 31 : lane == 0) ? 0.f : e;
}

template <int KIND, int LO>
__device__ __forceinline__ float interior_x(const float* w, int k, const WarpOp& p) {
#define W_(d) w[k + LO + (d)]
  if constexpr (KIND == K_DER1) {
    return p.ca * (W_(1) - W_(-1)) + p.cb * (W_(2) - W_(-2));
  } else {
    const float ur = W_(0);
    float acc = p.ca * (W_(1) - ur - ur + W_(-1)) + p.cb * (W_(2) - ur - ur + W_(-2));
    if (p.nterms_int > 2) acc = acc + p.cc * (W_(3) - ur - ur + W_(-3)) + p.cd * (W_(4) - ur - ur + W_(-4));
    return acc;
  }
#undef W_
}

// Solve of lane t's chunk of the warp's line; w[j] = u[t*L - LO + j].
template <int KIND, int L>
__device__ __forceinline__ void warp_solve(const float* w, float* v, const WarpOp& p, int lane) {
  constexpr int LO = Halo<KIND>::lo;
  const int r0 = lane * L;
  const int mode = p.mode[lane];
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = interior_x<KIND, LO>(w, k, p);
  float y = 0.f;
  if (mode & 1) {
#pragma unroll
    for (int k = 0; k < L; ++k) { y = v[k] - p.s_inf * y; v[k] = y; }
  } else {
#pragma unroll
    for (int k = 0; k < L; ++k) { y = v[k] - p.s[r0 + k] * y; v[k] = y; }
  }
  float cin = carry_scan<false>(p.pfe[lane], y, lane);
  // fix-up factors of this chunking (L rows) as running products
  if (mode & 1) {
    const float m = -p.s_inf;
    float P = m;
#pragma unroll
    for (int k = 0; k < L; ++k) { v[k] = v[k] + P * cin; P = P * m; }
  } else {
    float P = 1.f;
#pragma unroll
    for (int k = 0; k < L; ++k) { P = P * (-p.s[r0 + k]); v[k] = v[k] + P * cin; }
  }
  float x = 0.f;
  if (mode & 1) {
#pragma unroll
    for (int k = L - 1; k >= 0; --k) { x = (v[k] - p.f_inf * x) * p.w_inf; v[k] = x; }
  } else {
#pragma unroll
    for (int k = L - 1; k >= 0; --k) { x = (v[k] - p.f[r0 + k] * x) * p.w[r0 + k]; v[k] = x; }
  }
  cin = carry_scan<true>(p.qbs[lane], x, lane);
  if (mode & 1) {
    float Q = p.g_inf;
#pragma unroll
    for (int k = L - 1; k >= 0; --k) { v[k] = v[k] + Q * cin; Q = Q * p.g_inf; }
  } else {
    float Q = 1.f;
#pragma unroll
    for (int k = L - 1; k >= 0; --k) { Q = Q * (-(p.f[r0 + k] * p.w[r0 + k])); v[k] = v[k] + Q * cin; }
  }
  const float t1 = __shfl_sync(0xffffffffu, v[0], 0);
  const float tn = __shfl_sync(0xffffffffu, v[L - 1], 31);
  if (mode & 2) {
    const float sx = (t1 - p.alpha * tn) / p.den;
#pragma unroll
    for (int k = 0; k < L; ++k) v[k] = v[k] - sx * p.rsm[r0 + k];
  }
}

// Padded shared-memory index: lane t reading row t*L + j hits bank
// (t*L + j + (t*L + j)/32) mod 32, distinct over the warp for L = 4, 8, 16.
__device__ __forceinline__ int xpad(int r) { return r + (r >> 5); }

// Asynchronous 4-byte global -> shared copy (LDGSTS): the copies of a whole
// line are in flight at once and hold no registers.
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// Shared memory per warp: u_q, u_j and the running sum a1, each a padded line.
template <int L>
__host__ __device__ constexpr int xline_pad() {
  return 32 * L + L;
}

template <int L>
__global__ void __launch_bounds__(256, 3) rhs_fast_x(const __grid_constant__ RhsXArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 32 * L, NP = xline_pad<L>();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int line = blockIdx.x * 8 + warp;
  if (line >= p.na) return;  // whole warps only: the shuffles stay converged
  float* sq = reinterpret_cast<float*>(smem_raw) + (size_t)warp * 3 * NP;
  float* sa = sq + NP;
  float* s1 = sa + NP;
  const long long off = (long long)line * p.sa + (long long)blockIdx.y * p.sb;
  // line r = lane + 32 i goes to padded row r + i; group 0 = u_q and u_j,
  // group 1 = a1 (waited for only before the store)
  {
    const float* gq = p.uq + off;
    const float* ga = p.ua + off;
#pragma unroll
    for (int i = 0; i < L; ++i) {
      cp_async4(sq + lane + 33 * i, gq + lane + 32 * i);
      cp_async4(sa + lane + 33 * i, ga + lane + 32 * i);
    }
    cp_async_commit();
    if (p.a1) {
      const float* g1 = p.a1 + off;
#pragma unroll
      for (int i = 0; i < L; ++i) cp_async4(s1 + lane + 33 * i, g1 + lane + 32 * i);
    }
    cp_async_commit();
  }
  cp_async_wait<1>();
  __syncwarp();
  const int r0 = lane * L;
  const bool edge = (lane == 0 || lane == 31);
  float v[L], cv[L];
  {
    float w[L + 4];
#pragma unroll
    for (int j = 0; j < L + 4; ++j) {
      const int r = xpad(wrow(r0 - 2 + j, N, edge));
      w[j] = sq[r] * sa[r];
    }
    warp_solve<K_DER1, L>(w, v, p.A, lane);
  }
#pragma unroll
  for (int k = 0; k < L; ++k) cv[k] = v[k];
  {
    float w[L + 4];
#pragma unroll
    for (int j = 0; j < L + 4; ++j) w[j] = sq[xpad(wrow(r0 - 2 + j, N, edge))];
    warp_solve<K_DER1, L>(w, v, p.B, lane);
  }
#pragma unroll
  for (int k = 0; k < L; ++k) cv[k] = cv[k] + sa[xpad(r0 + k)] * v[k];
  {
    float w[L + 8];
#pragma unroll
    for (int j = 0; j < L + 8; ++j) w[j] = sq[xpad(wrow(r0 - 4 + j, N, edge))];
    warp_solve<K_DER2, L>(w, v, p.C, lane);
  }
  cp_async_wait<0>();
  __syncwarp();
#pragma unroll
  for (int k = 0; k < L; ++k) {
    sq[xpad(r0 + k)] = p.nu * v[k];
    sa[xpad(r0 + k)] = cv[k];
  }
  __syncwarp();
  // coalesced store: out = (nu C + a1) + (-1/2) conv
  float* dst = p.out + off;
  const bool has_a1 = p.a1 != nullptr;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    const int r = lane + 33 * i;
    float o = sq[r];
    if (has_a1) o = o + s1[r];
    o = o + (-0.5f) * sa[r];
    dst[lane + 32 * i] = o;
  }
}

void fill_warp_op(const OpPlan* p, WarpOp& a) {
  const int n = p->nout;
  const int L = n / XCH;
  const float* dv = p->dev32;
  a.s = dv; a.f = dv + n; a.w = dv + 2 * n; a.pf = dv + 3 * n; a.qb = dv + 4 * n; a.rsm = dv + 5 * n;
  a.ca = (float)p->ca; a.cb = (float)p->cb; a.cc = (float)p->cc; a.cd = (float)p->cd;
  a.alpha = (float)p->alpha;
  a.den = (float)p->den;
  a.nterms_int = (p->kind == K_DER2 && p->cc == 0.0 && p->cd == 0.0) ? 2 : 4;
  const int mid = n / 2;
  a.s_inf = (float)p->s[mid];
  a.f_inf = (float)p->f[mid];
  a.w_inf = (float)p->w[mid];
  a.g_inf = (float)(-(p->f[mid] * p->w[mid]));
  // chunk fix-up factors for chunks of L rows (the plan's are for n/16)
  for (int c = 0; c < XCH; ++c) {
    const int s0 = c * L, e0 = s0 + L - 1;
    double pe = 1.0, qs = 1.0;
    for (int r = s0; r <= e0; ++r) pe = pe * (-p->s[r]);
    for (int r = e0; r >= s0; --r) qs = qs * (-(p->f[r] * p->w[r]));
    a.pfe[c] = (float)pe;
    a.qbs[c] = (float)qs;
    bool uni = true, sm = false;
    for (int r = s0; r <= e0; ++r) {
      uni = uni && (float)p->s[r] == a.s_inf && (float)p->f[r] == a.f_inf && (float)p->w[r] == a.w_inf;
      sm = sm || (float)p->rsm[r] != 0.0f;
    }
    a.mode[c] = (uni ? 1 : 0) | (sm ? 2 : 0);
  }
}

template <bool XL, int L>
int launch_rhs_k(const RhsArgs& a, dim3 grid, size_t smem, cudaStream_t st) {
  auto kern = rhs_fast<XL, L>;
  static size_t configured = 0;
  if (smem > configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    configured = smem;
  }
  kern<<<grid, dim3(LANES, FCHUNKS), smem, st>>>(a);
  return cuda_status(cudaGetLastError());
}

template <int L>
int launch_rhs_x(const RhsXArgs& x, dim3 g, cudaStream_t st) {
  const size_t sm = (size_t)8 * 3 * xline_pad<L>() * sizeof(float);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(rhs_fast_x<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  rhs_fast_x<L><<<g, 256, sm, st>>>(x);
  return cuda_status(cudaGetLastError());
}

}  // namespace lk

using namespace lk;

static bool fast_line(const Ctx* c, const OpPlan* p) {
  return c->fast_lines && p->periodic && p->nin == p->nout && p->nout % FCHUNKS == 0 &&
         (p->nout / FCHUNKS == 8 || p->nout / FCHUNKS == 16 || p->nout / FCHUNKS == 32);
}

int rhs_axis_fast(Ctx* c, OpPlan* pA, OpPlan* pB, OpPlan* pC, float* out, const float* ua, const float* uq,
                  const float* a1, float nu, const int* dims, cudaStream_t st) {
  if (!fast_line(c, pA) || !fast_line(c, pB) || !fast_line(c, pC)) return X3D_ERR_UNSUPPORTED;
  const int axis = pA->axis;
  if (pB->axis != axis || pC->axis != axis || pA->kind != K_DER1 || pB->kind != K_DER1 || pC->kind != K_DER2)
    return X3D_ERR_ARG;
  for (OpPlan* p : {pA, pB, pC}) {
    const int up = upload_plan(p);
    if (up != X3D_OK) return up;
  }
  const int n = pA->nout;
  if (dims[axis] != n) return X3D_ERR_SHAPE;
  const int L = n / FCHUNKS;
  RhsArgs a;
  std::memset(&a, 0, sizeof(a));
  a.ua = ua;
  a.uq = uq;
  a.a1 = a1;
  a.out = out;
  a.n = n;
  a.nu = nu;
  dim3 grid;
  fast_geometry(axis, n, dims, &a.sa, &a.sb, &a.rs, &a.na, &grid);
  if (grid.y > 65535) return X3D_ERR_UNSUPPORTED;
  fill_fast_op(pA, a.A);
  fill_fast_op(pB, a.B);
  fill_fast_op(pC, a.C);
  const bool xl = (axis == 0);
  if (xl && n % XCH == 0 && (n / XCH == 4 || n / XCH == 8 || n / XCH == 16)) {
    RhsXArgs x;
    std::memset(&x, 0, sizeof(x));
    x.ua = ua; x.uq = uq; x.a1 = a1; x.out = out;
    x.n = n; x.na = a.na; x.sa = a.sa; x.sb = a.sb; x.nu = nu;
    fill_warp_op(pA, x.A);
    fill_warp_op(pB, x.B);
    fill_warp_op(pC, x.C);
    const dim3 g((unsigned)((a.na + 7) / 8), grid.y);
    const int Lx = n / XCH;
    if (Lx == 4) return launch_rhs_x<4>(x, g, st);
    if (Lx == 8) return launch_rhs_x<8>(x, g, st);
    return launch_rhs_x<16>(x, g, st);
  }
  const size_t base = (size_t)2 * FCHUNKS * LANES + 2 * LANES;
  const size_t smem = sizeof(float) * (base + (xl ? (size_t)2 * n * LD : (size_t)L * LANES * FCHUNKS));
  if (smem > 227 * 1024) return X3D_ERR_UNSUPPORTED;
  if (xl) {
    if (L == 8) return launch_rhs_k<true, 8>(a, grid, smem, st);
    if (L == 16) return launch_rhs_k<true, 16>(a, grid, smem, st);
    return launch_rhs_k<true, 32>(a, grid, smem, st);
  }
  if (L == 8) return launch_rhs_k<false, 8>(a, grid, smem, st);
  if (L == 16) return launch_rhs_k<false, 16>(a, grid, smem, st);
  return launch_rhs_k<false, 32>(a, grid, smem, st);
}

}  // namespace x3d
