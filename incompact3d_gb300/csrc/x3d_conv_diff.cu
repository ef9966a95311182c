// Fused momentum right-hand side along one axis (binary32, periodic lines).
//
// For one velocity component u_q and one direction j the reference forms, with
// transposes between the stages (src/transeq.f90:73-591),
//   conv_j = d_j(u_j u_q) + u_j d_j u_q,      visc_j = d_jj u_q,
// and sums them into the right-hand side.  Here one kernel runs the three
// compact solves of a line back to back:
//   out = (nu C(u_q) + a1) - (A(u_j u_q) + u_j B(u_q)) / 2
// so u_j, u_q and the running sum a1 are read from HBM once and out is written
// once (4 field passes instead of 11 with one kernel per solve).
//
// Periodic solves in circulant form.  On a periodic line the compact matrix
// of every operator here is circulant, A = I + alpha (S + S^-1) with S the
// cyclic shift, and factors exactly as
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
#include <cmath>

#include "x3d_line_fast.cuh"

namespace x3d {
namespace lk {

// One periodic compact operator in circulant form (binary32).
struct CircOp {
  float c1, c2, c3, c4;  // interior stencil coefficients times (1 + mu^2)
  float nmu;             // -mu
  int nterms;            // second derivative: 2 or 4 stencil terms
  int J;                 // chunk carries that reach binary32 (block kernel)
  float Ach;             // (-mu)^L: carry multiplier across one chunk
  float ak[5];           // Ach^(2^s): cyclic warp scan, s = 0..4
  float pw[32];          // (-mu)^(k+1): forward fix-up of chunk row k
  float qw[32];          // (-mu)^(L-k): backward fix-up of chunk row k
};

// Interior stencil (right-hand side B u) on the window w, w[j] = u[r0 - LO + j].
template <int KIND, int LO>
__device__ __forceinline__ float circ_rhs(const float* w, int k, const CircOp& p) {
#define W_(d) w[k + LO + (d)]
  if constexpr (KIND == K_DER1) {
    return p.c1 * (W_(1) - W_(-1)) + p.c2 * (W_(2) - W_(-2));
  } else {
    const float ur = W_(0);
    float acc = p.c1 * (W_(1) - ur - ur + W_(-1)) + p.c2 * (W_(2) - ur - ur + W_(-2));
    if (p.nterms > 2) acc = acc + p.c3 * (W_(3) - ur - ur + W_(-3)) + p.c4 * (W_(4) - ur - ur + W_(-4));
    return acc;
  }
#undef W_
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

// Block solve: thread (lane, ch) owns rows ch*L .. ch*L+L-1 of line `lane`;
// FC chunks per line, carries through shared memory (ef / eb: [FC][32]).
// Two block barriers; every thread of the block must call it.
template <int KIND, int L, int FC>
__device__ __forceinline__ void circ_block(const float* w, float* v, const CircOp& p, float* ef, float* eb, int ch,
                                           int lane) {
  constexpr int LO = Halo<KIND>::lo;
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = circ_rhs<KIND, LO>(w, k, p);
#pragma unroll
  for (int k = 1; k < L; ++k) v[k] = fmaf(p.nmu, v[k - 1], v[k]);
  ef[ch * 32 + lane] = v[L - 1];
  __syncthreads();
  float c = 0.f;
  for (int j = p.J; j >= 1; --j) c = fmaf(p.Ach, c, ef[((ch - j) & (FC - 1)) * 32 + lane]);
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = fmaf(p.pw[k], c, v[k]);
#pragma unroll
  for (int k = L - 2; k >= 0; --k) v[k] = fmaf(p.nmu, v[k + 1], v[k]);
  eb[ch * 32 + lane] = v[0];
  __syncthreads();
  c = 0.f;
  for (int j = p.J; j >= 1; --j) c = fmaf(p.Ach, c, eb[((ch + j) & (FC - 1)) * 32 + lane]);
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = fmaf(p.qw[k], c, v[k]);
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

struct CdArgs {
  const float *ua, *uq, *a1;  // u_j, u_q, running sum (may be null / alias out)
  float* out;
  long long sa, sb;  // line and plane offsets of the line (a, b)
  int rs;            // row stride (y/z lines)
  int na;            // lines per plane
  CircOp A, B, C;    // d(u_j u_q), d(u_q), dd(u_q)
  float nu;
};

// ---- x lines: one warp per line -------------------------------------------
// The line is contiguous: a warp stages it (u_q, u_j with a 4-row periodic
// halo at each end, and a1) into its own padded shared buffers with cp.async,
// then lane t solves rows t*L .. t*L+L-1 from there.  Row r lives at
//   P(r + L),  P(s) = s + floor(s / L),
// so the window of lane t is (L+1)(t+1) + d + floor(d/L) for row t*L + d:
// compile-time offsets from one base, and a stride of L+1 (odd) across the
// lanes, free of bank conflicts.
template <int L>
__host__ __device__ constexpr int xbuf() {
  return 32 * L + L + 40;
}
template <int L>
__device__ __forceinline__ constexpr int hoff(int d) {
  return d + (d >= 0 ? d / L : -1);  // -L <= d < 2L
}

template <int L>
__global__ void __launch_bounds__(256, 3) conv_diff_x(const __grid_constant__ CdArgs p) {
  extern __shared__ __align__(16) float smx[];
  constexpr int N = 32 * L, NB = xbuf<L>(), STEP = 32 + 32 / L;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int line = blockIdx.x * 8 + warp;
  if (line >= p.na) return;  // whole warps only: the shuffles stay converged
  float* sq = smx + (size_t)warp * 3 * NB;
  float* sa = sq + NB;
  float* s1 = sa + NB;
  const long long off = (long long)line * p.sa + (long long)blockIdx.y * p.sb;
  const int st0 = lane + lane / L + L + 1;  // P(lane + L)
  {
    const float* gq = p.uq + off;
    const float* ga = p.ua + off;
#pragma unroll
    for (int i = 0; i < L; ++i) {
      cp_async4(sq + st0 + i * STEP, gq + lane + 32 * i);
      cp_async4(sa + st0 + i * STEP, ga + lane + 32 * i);
    }
    if (lane < 8) {  // halo rows -4..-1 <- N-4..N-1 and N..N+3 <- 0..3
      const int g = (lane < 4) ? N - 4 + lane : lane - 4;
      const int d = (lane < 4) ? L - 4 + lane : N + L + 33 + (lane - 4);
      cp_async4(sq + d, gq + g);
      cp_async4(sa + d, ga + g);
    }
    cp_async_commit();
    if (p.a1) {
      const float* g1 = p.a1 + off;
#pragma unroll
      for (int i = 0; i < L; ++i) cp_async4(s1 + st0 + i * STEP, g1 + lane + 32 * i);
    }
    cp_async_commit();
  }
  cp_async_wait<1>();
  __syncwarp();
  const float* bq = sq + (L + 1) * (lane + 1);
  const float* ba = sa + (L + 1) * (lane + 1);
  float vB[L], v[L];
  {
    float wq[L + 8];  // u_q rows -4 .. L+3 of this lane's chunk
#pragma unroll
    for (int j = 0; j < L + 8; ++j) wq[j] = bq[hoff<L>(j - 4)];
    circ_warp<K_DER1, L>(wq + 2, vB, p.B, lane);
    circ_warp<K_DER2, L>(wq, v, p.C, lane);
  }
  cp_async_wait<0>();
  __syncwarp();
  float* b1 = s1 + (L + 1) * (lane + 1);
  if (p.a1) {
#pragma unroll
    for (int k = 0; k < L; ++k) b1[k] = __fadd_rn(__fmul_rn(p.nu, v[k]), b1[k]);
  } else {
#pragma unroll
    for (int k = 0; k < L; ++k) b1[k] = __fmul_rn(p.nu, v[k]);
  }
  {
    float w[L + 4];  // (u_j u_q) rows -2 .. L+1
#pragma unroll
    for (int j = 0; j < L + 4; ++j) w[j] = bq[hoff<L>(j - 2)] * ba[hoff<L>(j - 2)];
    circ_warp<K_DER1, L>(w, v, p.A, lane);
  }
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = fmaf(ba[k], vB[k], v[k]);  // conv = A + u_j B
  __syncwarp();  // every lane has read its windows of sq / sa
  float* bo = sa + (L + 1) * (lane + 1);
#pragma unroll
  for (int k = 0; k < L; ++k) bo[k] = v[k];
  __syncwarp();
  float* dst = p.out + off;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    const int s = st0 + i * STEP;
    dst[lane + 32 * i] = fmaf(-0.5f, sa[s], s1[s]);
  }
}

// ---- y / z lines: one thread per line across x, FC chunks per line --------
// Block (32 lanes, FC chunks): lane = line (32 consecutive x: one coalesced
// 128-byte segment per row), chunk ch = rows ch*L .. ch*L+L-1 of the line.
// Windows come straight from HBM / L2 into registers (u_q is read once per
// solve: the second and third reads hit L1 / L2); a1 is prefetched into
// shared memory with cp.async at the start; B(u_q) waits in shared memory
// while C and A are solved.
template <int WN, int N>
__device__ __forceinline__ void yz_window(float* w, const float* src, int r0m, int rs, bool edge) {
  if (edge) {
#pragma unroll
    for (int j = 0; j < WN; ++j) {
      int r = r0m + j;
      r = (r < 0) ? r + N : ((r >= N) ? r - N : r);
      w[j] = src[r * rs];
    }
  } else {
    const float* s = src + r0m * rs;
#pragma unroll
    for (int j = 0; j < WN; ++j) w[j] = s[j * rs];
  }
}

template <int WN, int N>
__device__ __forceinline__ void yz_window_prod(float* w, const float* src, const float* src2, int r0m, int rs,
                                               bool edge) {
  if (edge) {
#pragma unroll
    for (int j = 0; j < WN; ++j) {
      int r = r0m + j;
      r = (r < 0) ? r + N : ((r >= N) ? r - N : r);
      w[j] = src[r * rs] * src2[r * rs];
    }
  } else {
    const float* s = src + r0m * rs;
    const float* s2 = src2 + r0m * rs;
#pragma unroll
    for (int j = 0; j < WN; ++j) w[j] = s[j * rs] * s2[j * rs];
  }
}

template <int L, int FC>
__host__ __device__ constexpr size_t yz_smem() {
  return sizeof(float) * ((size_t)2 * L * 32 * FC + 2 * 32 * FC);
}

template <int L, int FC>
__global__ void __launch_bounds__(32 * FC, (FC >= 32) ? 1 : 2) conv_diff_yz(const __grid_constant__ CdArgs p) {
  extern __shared__ __align__(16) float smy[];
  constexpr int N = L * FC, NT = 32 * FC;
  float* stash = smy;           // [L][NT]: B(u_q)
  float* s1 = stash + L * NT;   // [L][NT]: a1, then nu C + a1
  float* ef = s1 + L * NT;      // [FC][32]
  float* eb = ef + 32 * FC;     // [FC][32]
  const int lane = threadIdx.x, ch = threadIdx.y, tid = ch * 32 + lane;
  const int a0 = blockIdx.x * 32;
  const bool ok = a0 + lane < p.na;
  // lanes past the last line solve line a0 (valid memory) and store nothing
  const long long base = (long long)(ok ? a0 + lane : a0) * p.sa + (long long)blockIdx.y * p.sb;
  const int rs = p.rs, r0 = ch * L;
  const bool edge = (ch == 0 || ch == FC - 1);
  const float* q = p.uq + base;
  const float* ua = p.ua + base;
  if (p.a1) {
    const float* g1 = p.a1 + base + (long long)r0 * rs;
#pragma unroll
    for (int k = 0; k < L; ++k) cp_async4(s1 + k * NT + tid, g1 + k * rs);
  }
  cp_async_commit();
  float v[L];
  {
    float wq[L + 4];  // u_q rows r0-2 .. r0+L+1
    yz_window<L + 4, N>(wq, q, r0 - 2, rs, edge);
    circ_block<K_DER1, L, FC>(wq, v, p.B, ef, eb, ch, lane);
  }
#pragma unroll
  for (int k = 0; k < L; ++k) stash[k * NT + tid] = v[k];
  {
    float wq[L + 8];  // u_q rows r0-4 .. r0+L+3 (again: L1 / L2 hits)
    yz_window<L + 8, N>(wq, q, r0 - 4, rs, edge);
    circ_block<K_DER2, L, FC>(wq, v, p.C, ef, eb, ch, lane);
  }
  cp_async_wait<0>();  // own entries only: no barrier needed
  if (p.a1) {
#pragma unroll
    for (int k = 0; k < L; ++k) s1[k * NT + tid] = __fadd_rn(__fmul_rn(p.nu, v[k]), s1[k * NT + tid]);
  } else {
#pragma unroll
    for (int k = 0; k < L; ++k) s1[k * NT + tid] = __fmul_rn(p.nu, v[k]);
  }
  {
    float w[L + 4];  // (u_j u_q) rows r0-2 .. r0+L+1
    yz_window_prod<L + 4, N>(w, q, ua, r0 - 2, rs, edge);
    circ_block<K_DER1, L, FC>(w, v, p.A, ef, eb, ch, lane);
  }
  if (ok) {
    const float* uj = ua + (long long)r0 * rs;
    float* dst = p.out + base + (long long)r0 * rs;
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const float conv = fmaf(uj[k * rs], stash[k * NT + tid], v[k]);  // A + u_j B
      dst[k * rs] = fmaf(-0.5f, conv, s1[k * NT + tid]);
    }
  }
}

// ---- host side -------------------------------------------------------------
// Circulant form of a periodic plan for chunks of L rows.
static int fill_circ(const OpPlan* p, int L, int max_carries, CircOp& c) {
  if (!p->periodic || p->nin != p->nout || (p->kind != K_DER1 && p->kind != K_DER2)) return X3D_ERR_UNSUPPORTED;
  const double al = p->alpha;
  if (!(4.0 * al * al < 1.0)) return X3D_ERR_UNSUPPORTED;  // not diagonally dominant
  const double mu = 2.0 * al / (1.0 + std::sqrt(1.0 - 4.0 * al * al));
  const double sc = 1.0 + mu * mu;
  std::memset(&c, 0, sizeof(c));
  c.c1 = (float)(p->ca * sc);
  c.c2 = (float)(p->cb * sc);
  c.c3 = (float)(p->cc * sc);
  c.c4 = (float)(p->cd * sc);
  c.nterms = (p->kind == K_DER2 && p->cc == 0.0 && p->cd == 0.0) ? 2 : 4;
  c.nmu = (float)(-mu);
  const double A = std::pow(-mu, L);
  c.Ach = (float)A;
  double a = A;
  for (int s = 0; s < 5; ++s) {
    c.ak[s] = (float)a;
    a = a * a;
  }
  for (int k = 0; k < 32; ++k) {
    c.pw[k] = (k < L) ? (float)std::pow(-mu, k + 1) : 0.f;
    c.qw[k] = (k < L) ? (float)std::pow(-mu, L - k) : 0.f;
  }
  // carries whose weight |A|^(j-1) stays above 2^-32 of the nearest one
  int J = 1;
  const double lim = std::ldexp(1.0, -32);
  for (double w = std::fabs(A); J < max_carries && w >= lim; w *= std::fabs(A)) ++J;
  if (std::pow(std::fabs(A), J) >= lim) return X3D_ERR_UNSUPPORTED;  // the scan would wrap onto itself
  c.J = J;
  return X3D_OK;
}

template <int L>
static int launch_cd_x(const CdArgs& a, dim3 g, cudaStream_t st) {
  const size_t sm = (size_t)8 * 3 * xbuf<L>() * sizeof(float);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(conv_diff_x<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  conv_diff_x<L><<<g, 256, sm, st>>>(a);
  return cuda_status(cudaGetLastError());
}

template <int L, int FC>
static int launch_cd_yz(const CdArgs& a, dim3 g, cudaStream_t st) {
  constexpr size_t sm = yz_smem<L, FC>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(conv_diff_yz<L, FC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  conv_diff_yz<L, FC><<<g, dim3(32, FC), sm, st>>>(a);
  return cuda_status(cudaGetLastError());
}

// Chunking of a line of n rows: x lines one warp (L = n/32), y/z lines FC
// chunks of L rows.  Returns false where no kernel is instantiated.
static bool cd_shape(int axis, int n, int* L, int* FC) {
  if (axis == 0) {
    if (n != 128 && n != 256 && n != 512) return false;
    *L = n / 32;
    *FC = 32;
    return true;
  }
  if (n == 128) { *L = 8; *FC = 16; return true; }
  if (n == 256) { *L = 16; *FC = 16; return true; }
  if (n == 512) { *L = 16; *FC = 32; return true; }
  return false;
}

}  // namespace lk

using namespace lk;

bool rhs_axis_fast_ok(const Ctx* c, int axis, const int* dims) {
  int L, FC;
  if (!c->fast_lines || !c->ax[axis].periodic || !cd_shape(axis, dims[axis], &L, &FC)) return false;
  if (axis == 1 && c->st.istret != 0) return false;
  const long long rs = (axis == 0) ? 1 : (axis == 1 ? (long long)dims[0] : (long long)dims[0] * dims[1]);
  return (long long)dims[axis] * rs < (1LL << 31);
}

int rhs_axis_fast(Ctx* c, OpPlan* pA, OpPlan* pB, OpPlan* pC, float* out, const float* ua, const float* uq,
                  const float* a1, float nu, const int* dims, cudaStream_t st) {
  const int axis = pA->axis;
  if (pB->axis != axis || pC->axis != axis || pA->kind != K_DER1 || pB->kind != K_DER1 || pC->kind != K_DER2)
    return X3D_ERR_ARG;
  if (!rhs_axis_fast_ok(c, axis, dims)) return X3D_ERR_UNSUPPORTED;
  const int n = dims[axis];
  if (pA->nout != n || pB->nout != n || pC->nout != n) return X3D_ERR_SHAPE;
  int L = 0, FC = 0;
  cd_shape(axis, n, &L, &FC);
  CdArgs a;
  std::memset(&a, 0, sizeof(a));
  a.ua = ua;
  a.uq = uq;
  a.a1 = a1;
  a.out = out;
  a.nu = nu;
  int rc = fill_circ(pA, L, axis == 0 ? 32 : FC - 1, a.A);
  if (rc == X3D_OK) rc = fill_circ(pB, L, axis == 0 ? 32 : FC - 1, a.B);
  if (rc == X3D_OK) rc = fill_circ(pC, L, axis == 0 ? 32 : FC - 1, a.C);
  if (rc != X3D_OK) return rc;
  const long long nx = dims[0], ny = dims[1], nz = dims[2];
  if (axis == 0) {
    // warp per x line: lines (j, k) with j in a block of 8, k = blockIdx.y
    a.na = (int)ny;
    a.sa = nx;
    a.sb = nx * ny;
    a.rs = 1;
    if (nz > 65535) return X3D_ERR_UNSUPPORTED;
    const dim3 g((unsigned)((ny + 7) / 8), (unsigned)nz);
    if (L == 4) return launch_cd_x<4>(a, g, st);
    if (L == 8) return launch_cd_x<8>(a, g, st);
    return launch_cd_x<16>(a, g, st);
  }
  // y lines: (i, k), z lines: (i, j); 32 consecutive i per block
  a.na = (int)nx;
  a.sa = 1;
  a.sb = (axis == 1) ? nx * ny : nx;
  a.rs = (int)((axis == 1) ? nx : nx * ny);
  const long long planes = (axis == 1) ? nz : ny;
  if (planes > 65535) return X3D_ERR_UNSUPPORTED;
  const dim3 g((unsigned)((nx + 31) / 32), (unsigned)planes);
  if (L == 8) return launch_cd_yz<8, 16>(a, g, st);
  if (FC == 16) return launch_cd_yz<16, 16>(a, g, st);
  return launch_cd_yz<16, 32>(a, g, st);
}

}  // namespace x3d
