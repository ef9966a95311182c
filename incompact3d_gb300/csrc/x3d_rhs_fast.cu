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
#pragma unroll
      for (int j = 0; j < W1; ++j) {
        const long long r = wrow(r0 - 2 + j, n, edge);
        w[j] = ok ? q[r * p.rs] * ua[r * p.rs] : 0.f;
      }
      fast_solve<float, K_DER1, L>(w, v, p.A, cfw, cbw, ends, ch, lane);
    }
#pragma unroll
    for (int k = 0; k < L; ++k) stash[k * NT + tid] = v[k];
    {
      float w[W1];
#pragma unroll
      for (int j = 0; j < W1; ++j) {
        const long long r = wrow(r0 - 2 + j, n, edge);
        w[j] = ok ? q[r * p.rs] : 0.f;
      }
      fast_solve<float, K_DER1, L>(w, v, p.B, cfw, cbw, ends, ch, lane);
    }
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const float uj = ok ? ua[(long long)(r0 + k) * p.rs] : 0.f;
      stash[k * NT + tid] = stash[k * NT + tid] + uj * v[k];
    }
    {
      float w[W2];
#pragma unroll
      for (int j = 0; j < W2; ++j) {
        const long long r = wrow(r0 - 4 + j, n, edge);
        w[j] = ok ? q[r * p.rs] : 0.f;
      }
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
