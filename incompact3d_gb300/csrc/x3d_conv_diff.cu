// Fused momentum right-hand side along one axis (binary32, periodic lines).
//
// For one velocity component u_q and one direction j the reference forms, with
// transposes between the stages (src/transeq.f90:73-591),
//   conv_j = d_j(u_j u_q) + u_j d_j u_q,      visc_j = d_jj u_q,
// and sums them into the right-hand side.  Here one kernel runs the three
// compact solves of a line back to back:
//   out = (nu C(u_q) + a1) - (A(u_j u_q) + u_j B(u_q)) / 2
// so u_j, u_q and the running sum a1 are read from HBM once and out is written
// once (4 field passes instead of 11 with one kernel per solve).  The x kernel
// rounds in that order; the y/z kernel accumulates a1 + (nu C - A/2 - u_j B/2)
// (same terms, binary32 round-off apart).  The solves are in circulant form
// (x3d_circ.cuh).
#include <cmath>
#include <cstdint>

#include "x3d_circ.cuh"

namespace x3d {
namespace lk {

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
// then lane t solves rows t*L .. t*L+L-1 from there and stores its L
// contiguous results with 16-byte stores.  Row r lives at
//   P(r + L),  P(s) = s + floor(s / L),
// so the window of lane t is (L+1)(t+1) + d + floor(d/L) for row t*L + d:
// compile-time offsets from one base, and a stride of L+1 (odd) across the
// lanes, free of bank conflicts.

// Warps (lines) per block and blocks per SM: 4 x 5 = 20 warps, ~100 registers
// per thread for the three solves of L = 16 rows without spills.
constexpr int XW = 4, XB = 5;

template <int L>
__global__ void __launch_bounds__(32 * XW, XB) conv_diff_x(const __grid_constant__ CdArgs p) {
  extern __shared__ __align__(16) float smx[];
  constexpr int N = 32 * L, NB = xbuf<L>(), STEP = 32 + 32 / L;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int line = blockIdx.x * XW + warp;
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
  float conv[L], v[L];
  {
    float w[L + 4];  // A: d_j(u_j u_q), rows -2 .. L+1
#pragma unroll
    for (int j = 0; j < L + 4; ++j) w[j] = bq[hoff<L>(j - 2)] * ba[hoff<L>(j - 2)];
    circ_warp<K_DER1, L>(w, conv, p.A, lane);
  }
  float wq[L + 8];  // u_q rows -4 .. L+3 of this lane's chunk (B and C)
#pragma unroll
  for (int j = 0; j < L + 8; ++j) wq[j] = bq[hoff<L>(j - 4)];
  circ_warp<K_DER1, L>(wq + 2, v, p.B, lane);
#pragma unroll
  for (int k = 0; k < L; ++k) conv[k] = fmaf(ba[k], v[k], conv[k]);  // A + u_j B
  circ_warp<K_DER2, L>(wq, v, p.C, lane);
  cp_async_wait<0>();
  __syncwarp();
  // out = (nu C + a1) - conv / 2 for this lane's L contiguous rows (16-byte stores)
  const float* b1 = s1 + (L + 1) * (lane + 1);
  float4* dst = reinterpret_cast<float4*>(p.out + off + L * lane);
#pragma unroll
  for (int k4 = 0; k4 < L / 4; ++k4) {
    float o[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int k = 4 * k4 + m;
      float c = __fmul_rn(p.nu, v[k]);
      if (p.a1) c = __fadd_rn(c, b1[k]);
      o[m] = fmaf(-0.5f, conv[k], c);
    }
    dst[k4] = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// ---- y / z lines: two lines per thread, FC chunks per line -----------------
// Block: 8 column pairs (16 consecutive x lines) x FC chunks of L = 8 rows.
// The block first copies its slab of u_q and u_j (all N rows of its 16 lines
// plus 4 periodic halo rows at each end) into shared memory with 8-byte
// cp.async: every HBM load of the block is in flight at once, and two blocks
// per SM overlap one's copy with the other's solves.  A thread then reads its
// two lines as float2 (half the shared-memory instructions of one line per
// thread, and two independent recurrence chains).  The three results are
// accumulated in registers as r = nu C - A/2 - u_j B/2 (the solves in the
// order C, A, B) and out = a1 + r is written with a1 read in the epilogue.
// Slab row r (-4 <= r < N+4), line c sits at (r + 4) * 18 + c: the chunks of a
// half-warp (rows 8 apart: 8 * 18 = 16 mod 32 words) fall in disjoint banks.
template <int FC>
__host__ __device__ constexpr size_t yz_smem() {
  return sizeof(float) * ((size_t)2 * (YL * FC + 8) * SR2 + (size_t)4 * FC * CP);
}

template <int FC>
__global__ void __launch_bounds__(CP* FC, (CP * FC <= 512) ? 2 : 1) conv_diff_yz(const __grid_constant__ CdArgs p) {
  extern __shared__ __align__(16) float smy[];
  constexpr int L = YL, N = L * FC, NT = CP * FC, SLAB = (N + 8) * SR2;
  float* su = smy;
  float* sa = su + SLAB;
  float2* ef = reinterpret_cast<float2*>(sa + SLAB);
  float2* eb = ef + FC * CP;
  const int cp = threadIdx.x, ch = threadIdx.y, t = ch * CP + cp;
  const long long pb = (long long)blockIdx.y * p.sb + (long long)blockIdx.x * 2 * CP;
  const int rs = p.rs;
  {
    // float2 element e = t + NT i -> row e / 8, pair e % 8 (a warp copies four
    // 64-byte row segments per instruction)
#pragma unroll
    for (int i = 0; i < L; ++i) {
      const int e = t + NT * i;
      const int r = e >> 3, c = 2 * (e & 7);
      const long long g = pb + (long long)r * rs + c;
      const int d = (r + 4) * SR2 + c;
      cp_async8(su + d, p.uq + g);
      cp_async8(sa + d, p.ua + g);
    }
    if (t < 8 * CP) {  // halo rows -4..-1 <- N-4..N-1 and N..N+3 <- 0..3
      const int h = t >> 3, c = 2 * (t & 7);
      const int r = (h < 4) ? h - 4 : N + h - 4;
      const int rg = (h < 4) ? N - 4 + h : h - 4;
      const long long g = pb + (long long)rg * rs + c;
      const int d = (r + 4) * SR2 + c;
      cp_async8(su + d, p.uq + g);
      cp_async8(sa + d, p.ua + g);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
  }
  constexpr int R2 = SR2 / 2;  // slab row stride in float2
  const int o0 = ((ch * L + 4) * SR2 + 2 * cp) / 2;
  const float2* bu = reinterpret_cast<const float2*>(su) + o0;
  const float2* ba = reinterpret_cast<const float2*>(sa) + o0;
  float2 v[L], r[L];
  {
    float2 w[L + 8];  // C: d_jj u_q, rows r0-4 .. r0+L+3
#pragma unroll
    for (int j = 0; j < L + 8; ++j) w[j] = bu[(j - 4) * R2];
    circ_block2<K_DER2, L, FC>(w, v, p.C, ef, eb, ch, cp);
  }
#pragma unroll
  for (int k = 0; k < L; ++k) r[k] = make_float2(p.nu * v[k].x, p.nu * v[k].y);
  {
    float2 w[L + 4];  // A: d_j(u_j u_q), rows r0-2 .. r0+L+1
#pragma unroll
    for (int j = 0; j < L + 4; ++j) {
      const float2 q = bu[(j - 2) * R2], a = ba[(j - 2) * R2];
      w[j] = make_float2(q.x * a.x, q.y * a.y);
    }
    circ_block2<K_DER1, L, FC>(w, v, p.A, ef, eb, ch, cp);
  }
#pragma unroll
  for (int k = 0; k < L; ++k) r[k] = f2fma(-0.5f, v[k], r[k]);
  {
    float2 w[L + 4];  // B: d_j u_q
#pragma unroll
    for (int j = 0; j < L + 4; ++j) w[j] = bu[(j - 2) * R2];
    circ_block2<K_DER1, L, FC>(w, v, p.B, ef, eb, ch, cp);
  }
#pragma unroll
  for (int k = 0; k < L; ++k) {
    const float2 uj = ba[k * R2];
    r[k] = f2fma2(make_float2(-0.5f * uj.x, -0.5f * uj.y), v[k], r[k]);
  }
  // a1 may alias out: this thread reads its own rows of a1 before writing them
  const long long o = pb + 2 * cp + (long long)(ch * L) * rs;
  float2 a1v[L];
#pragma unroll
  for (int k = 0; k < L; ++k)
    a1v[k] = p.a1 ? *reinterpret_cast<const float2*>(p.a1 + o + (long long)k * rs) : make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < L; ++k)
    *reinterpret_cast<float2*>(p.out + o + (long long)k * rs) = make_float2(a1v[k].x + r[k].x, a1v[k].y + r[k].y);
}

// ---- host side -------------------------------------------------------------
// Circulant form of a periodic plan for chunks of L rows.
int fill_circ(const OpPlan* p, int L, int max_carries, CircOp& c) {
  if (!p->periodic || p->nin != p->nout) return X3D_ERR_UNSUPPORTED;
  const double al = p->alpha;
  if (!(4.0 * al * al < 1.0)) return X3D_ERR_UNSUPPORTED;  // not diagonally dominant
  if (!plan_is_circulant(p)) return X3D_ERR_UNSUPPORTED;
  const double mu = 2.0 * al / (1.0 + std::sqrt(1.0 - 4.0 * al * al));
  const double sc = 1.0 + mu * mu;
  std::memset(&c, 0, sizeof(c));
  c.c1 = (float)(p->ca * sc);
  c.c2 = (float)(p->cb * sc);
  c.c3 = (float)(p->cc * sc);
  c.c4 = (float)(p->cd * sc);
  c.nterms = 4;
  if (p->kind == K_DER2 && p->cc == 0.0 && p->cd == 0.0) c.nterms = 2;
  if ((p->kind == K_IVP || p->kind == K_IPV) && p->cd == 0.0) c.nterms = 3;
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
  const size_t sm = (size_t)XW * 3 * xbuf<L>() * sizeof(float);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(conv_diff_x<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  conv_diff_x<L><<<g, 32 * XW, sm, st>>>(a);
  return cuda_status(cudaGetLastError());
}

template <int FC>
static int launch_cd_yz(const CdArgs& a, dim3 g, cudaStream_t st) {
  constexpr size_t sm = yz_smem<FC>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(conv_diff_yz<FC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  conv_diff_yz<FC><<<g, dim3(CP, FC), sm, st>>>(a);
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
  if (n != 128 && n != 256 && n != 512) return false;
  *L = YL;
  *FC = n / YL;
  return true;
}

}  // namespace lk

using namespace lk;

bool rhs_axis_fast_ok(const Ctx* c, int axis, const int* dims) {
  int L, FC;
  if (!c->fast_lines || !c->ax[axis].periodic || !cd_shape(axis, dims[axis], &L, &FC)) return false;
  if (axis == 1 && c->st.istret != 0) return false;
  const long long rs = (axis == 0) ? 1 : (axis == 1 ? (long long)dims[0] : (long long)dims[0] * dims[1]);
  if (axis != 0 && dims[0] % (2 * CP) != 0) return false;  // y/z blocks: 16 whole x lines
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
    // warp per x line: lines (j, k) with j in a block of XW, k = blockIdx.y;
    // each lane stores its L rows as float4
    // each lane stores its L rows as float4
    if (reinterpret_cast<uintptr_t>(out) % 16 != 0) return X3D_ERR_UNSUPPORTED;
    a.na = (int)ny;
    a.sa = nx;
    a.sb = nx * ny;
    a.rs = 1;
    if (nz > 65535) return X3D_ERR_UNSUPPORTED;
    const dim3 g((unsigned)((ny + XW - 1) / XW), (unsigned)nz);
    if (L == 4) return launch_cd_x<4>(a, g, st);
    if (L == 8) return launch_cd_x<8>(a, g, st);
    return launch_cd_x<16>(a, g, st);
  }
  // y lines: (i, k), z lines: (i, j); 16 consecutive i per block
  a.na = (int)nx;
  a.sa = 1;
  a.sb = (axis == 1) ? nx * ny : nx;
  a.rs = (int)((axis == 1) ? nx : nx * ny);
  const long long planes = (axis == 1) ? nz : ny;
  if (planes > 65535) return X3D_ERR_UNSUPPORTED;
  // 8-byte copies and stores of line pairs
  if ((reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(ua) | reinterpret_cast<uintptr_t>(uq) |
       reinterpret_cast<uintptr_t>(a1)) % 8 != 0)
    return X3D_ERR_UNSUPPORTED;
  const dim3 g((unsigned)(nx / (2 * CP)), (unsigned)planes);
  if (FC == 16) return launch_cd_yz<16>(a, g, st);
  if (FC == 32) return launch_cd_yz<32>(a, g, st);
  return launch_cd_yz<64>(a, g, st);
}

}  // namespace x3d
