// Staggered divergence / gradient operators of the periodic binary32 step,
// in circulant form (x3d_circ.cuh) and fused per axis where the data flow of
// the reference allows.
//
// divergence (src/navier.f90:257-372) on a periodic grid:
//   x: pp1 = derxvp(ux), pgy1 = interxvp(uy), pgz1 = interxvp(uz)
//   y: duy = deryvp(pgy1) + interyvp(pp1)          (one kernel, two slabs)
//      upi2 = interyvp(pgz1)
//   z: pp3 = interzvp(duy) + derzvp(upi2)          (one kernel, FP64 output)
// gradp (src/navier.f90:386-432):
//   z: ppi3 = interzpv(pp3), pgz3 = derzpv(pp3)    (one kernel, one slab)
//   y: ppi2 = interypv(ppi3), pgy2 = derypv(ppi3)  (one kernel, one slab)
//      pgzi2 = interypv(pgz3)
//   x: px = derxpv(ppi2), py = interxpv(pgy2), pz = interxpv(pgzi2)
// The sums are formed in binary32 in the reference's order (A + B) before
// any conversion.  x lines: one warp per line (as conv_diff_x); y/z lines: a
// block stages the slab of its 16 lines with cp.async and a thread solves two
// lines of one chunk (as conv_diff_yz).
#include <cmath>
#include <cstdint>

#include "x3d_circ.cuh"
#include "x3d_df.cuh"

namespace x3d {
namespace lk {

enum { SM_ONE = 0, SM_SUM = 1, SM_DUAL = 2 };

struct StArgs {
  const float *in0, *in1;  // in1: second input (SUM)
  void* out0;              // float, or double for a SUM with FP64 output
  float* out1;             // second output (DUAL)
  long long sa, sb;        // line and plane offsets
  int rs, na;              // row stride (y/z), lines per plane
  CircOp A, B;
  float *ch, *cl;          // x lines: (ch, cl) -= result instead of writing out0
};

// ---- x lines: one warp per line, one solve -----------------------------------
constexpr int SXW = 8;  // warps (lines) per block

// COR: the correction mode (p.ch, p.cl set), a separate instantiation so the
// plain kernel keeps its register count.
template <int L, int K, bool COR>
__global__ void __launch_bounds__(32 * SXW) stag_x(const __grid_constant__ StArgs p) {
  extern __shared__ __align__(16) float sxm[];
  constexpr int N = 32 * L, NB = xbuf<L>(), STEP = 32 + 32 / L;
  constexpr int LO = Halo<K>::lo, HI = Halo<K>::hi;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int line = blockIdx.x * SXW + warp;
  if (line >= p.na) return;  // whole warps only
  float* sq = sxm + (size_t)warp * NB;
  const long long off = (long long)line * p.sa + (long long)blockIdx.y * p.sb;
  const int st0 = lane + lane / L + L + 1;
  // correction mode: this lane's L points of the state are loaded while the
  // line is staged, so their latency is not exposed after the solve
  float4 ch4[COR ? L / 4 : 1], cl4[COR ? L / 4 : 1];
  {
    const float* g = p.in0 + off;
#pragma unroll
    for (int i = 0; i < L; ++i) cp_async4(sq + st0 + i * STEP, g + lane + 32 * i);
    if (lane < 8) {  // halo rows -4..-1 <- N-4..N-1 and N..N+3 <- 0..3
      const int gi = (lane < 4) ? N - 4 + lane : lane - 4;
      const int d = (lane < 4) ? L - 4 + lane : N + L + 33 + (lane - 4);
      cp_async4(sq + d, g + gi);
    }
    cp_async_commit();
    if (COR) {
      const float4* hp = reinterpret_cast<const float4*>(p.ch + off + L * lane);
      const float4* lp = reinterpret_cast<const float4*>(p.cl + off + L * lane);
#pragma unroll
      for (int k4 = 0; k4 < L / 4; ++k4) {
        ch4[k4] = hp[k4];
        cl4[k4] = lp[k4];
      }
    }
    cp_async_wait<0>();
    __syncwarp();
  }
  const float* bq = sq + (L + 1) * (lane + 1);
  float w[L + LO + HI], v[L];
#pragma unroll
  for (int j = 0; j < L + LO + HI; ++j) w[j] = bq[hoff<L>(j - LO)];
  circ_warp<K, L>(w, v, p.A, lane);
  if (COR) {
    // pressure correction of a double-float velocity component (cor_vel):
    // the same two-sum update as a separate pass over the stored gradient
    float4* hp = reinterpret_cast<float4*>(p.ch + off + L * lane);
    float4* lp = reinterpret_cast<float4*>(p.cl + off + L * lane);
#pragma unroll
    for (int k4 = 0; k4 < L / 4; ++k4) {
      float4 h = ch4[k4], l = cl4[k4];
      df_add_f(h.x, l.x, -v[4 * k4]);
      df_add_f(h.y, l.y, -v[4 * k4 + 1]);
      df_add_f(h.z, l.z, -v[4 * k4 + 2]);
      df_add_f(h.w, l.w, -v[4 * k4 + 3]);
      hp[k4] = h;
      lp[k4] = l;
    }
    return;
  }
  float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(p.out0) + off + L * lane);
#pragma unroll
  for (int k4 = 0; k4 < L / 4; ++k4) dst[k4] = make_float4(v[4 * k4], v[4 * k4 + 1], v[4 * k4 + 2], v[4 * k4 + 3]);
}

// ---- y / z lines: two lines per thread ------------------------------------------
template <int FC, int NS>
__host__ __device__ constexpr size_t st_smem() {
  return sizeof(float) * ((size_t)NS * (YL * FC + 8) * SR2 + (size_t)4 * FC * CP);
}

template <int FC, int KA, int KB, int MODE, bool OUT64>
__global__ void __launch_bounds__(CP* FC, (CP * FC <= 512) ? 2 : 1) stag_yz(const __grid_constant__ StArgs p) {
  extern __shared__ __align__(16) float sym[];
  constexpr int L = YL, N = L * FC, NT = CP * FC, SLAB = (N + 8) * SR2;
  constexpr int NS = (MODE == SM_SUM) ? 2 : 1;
  float* s0 = sym;
  float* s1 = s0 + SLAB;  // SUM only
  float2* ef = reinterpret_cast<float2*>(sym + NS * SLAB);
  float2* eb = ef + FC * CP;
  const int cp = threadIdx.x, ch = threadIdx.y, t = ch * CP + cp;
  const long long pb = (long long)blockIdx.y * p.sb + (long long)blockIdx.x * 2 * CP;
  const int rs = p.rs;
  {
#pragma unroll
    for (int i = 0; i < L; ++i) {
      const int e = t + NT * i;
      const int r = e >> 3, c = 2 * (e & 7);
      const long long g = pb + (long long)r * rs + c;
      const int d = (r + 4) * SR2 + c;
      cp_async8(s0 + d, p.in0 + g);
      if (MODE == SM_SUM) cp_async8(s1 + d, p.in1 + g);
    }
    if (t < 8 * CP) {  // halo rows -4..-1 <- N-4..N-1 and N..N+3 <- 0..3
      const int h = t >> 3, c = 2 * (t & 7);
      const int r = (h < 4) ? h - 4 : N + h - 4;
      const int rg = (h < 4) ? N - 4 + h : h - 4;
      const long long g = pb + (long long)rg * rs + c;
      const int d = (r + 4) * SR2 + c;
      cp_async8(s0 + d, p.in0 + g);
      if (MODE == SM_SUM) cp_async8(s1 + d, p.in1 + g);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
  }
  constexpr int R2 = SR2 / 2;
  const int o0 = ((ch * L + 4) * SR2 + 2 * cp) / 2;
  float2* b0 = reinterpret_cast<float2*>(s0) + o0;
  const long long o = pb + 2 * cp + (long long)(ch * L) * rs;
  float2 v[L];
  {
    constexpr int LO = Halo<KA>::lo, HI = Halo<KA>::hi;
    float2 w[L + LO + HI];
#pragma unroll
    for (int j = 0; j < L + LO + HI; ++j) w[j] = b0[(j - LO) * R2];
    circ_block2<KA, L, FC>(w, v, p.A, ef, eb, ch, cp);
  }
  if (MODE != SM_SUM) {
    float* out = reinterpret_cast<float*>(p.out0);
#pragma unroll
    for (int k = 0; k < L; ++k) *reinterpret_cast<float2*>(out + o + (long long)k * rs) = v[k];
  }
  if (MODE == SM_DUAL) {
    constexpr int LO = Halo<KB>::lo, HI = Halo<KB>::hi;
    float2 w[L + LO + HI];
#pragma unroll
    for (int j = 0; j < L + LO + HI; ++j) w[j] = b0[(j - LO) * R2];
    circ_block2<KB, L, FC>(w, v, p.B, ef, eb, ch, cp);
#pragma unroll
    for (int k = 0; k < L; ++k) *reinterpret_cast<float2*>(p.out1 + o + (long long)k * rs) = v[k];
  }
  if (MODE == SM_SUM) {
    // every thread read its first window before the first barrier of the
    // solve: the own rows of the first slab now hold A
#pragma unroll
    for (int k = 0; k < L; ++k) b0[k * R2] = v[k];
    const float2* b1 = reinterpret_cast<const float2*>(s1) + o0;
    {
      constexpr int LO = Halo<KB>::lo, HI = Halo<KB>::hi;
      float2 w[L + LO + HI];
#pragma unroll
      for (int j = 0; j < L + LO + HI; ++j) w[j] = b1[(j - LO) * R2];
      circ_block2<KB, L, FC>(w, v, p.B, ef, eb, ch, cp);
    }
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const float2 a = b0[k * R2];
      const float sx = a.x + v[k].x, sy = a.y + v[k].y;
      if (OUT64) {
        *reinterpret_cast<double2*>(reinterpret_cast<double*>(p.out0) + o + (long long)k * rs) =
            make_double2((double)sx, (double)sy);
      } else {
        *reinterpret_cast<float2*>(reinterpret_cast<float*>(p.out0) + o + (long long)k * rs) = make_float2(sx, sy);
      }
    }
  }
}

// ---- host side -------------------------------------------------------------
template <typename KERN>
static int launch_dyn(KERN kern, dim3 g, dim3 b, size_t sm, cudaStream_t st, const StArgs& a, bool& configured) {
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  kern<<<g, b, sm, st>>>(a);
  return cuda_status(cudaGetLastError());
}

template <int L, int K>
static int run_x(const StArgs& a, dim3 g, cudaStream_t st) {
  static bool conf = false, conf_cor = false;
  const size_t sm = (size_t)SXW * xbuf<L>() * sizeof(float);
  if (a.ch) return launch_dyn(stag_x<L, K, true>, g, dim3(32 * SXW), sm, st, a, conf_cor);
  return launch_dyn(stag_x<L, K, false>, g, dim3(32 * SXW), sm, st, a, conf);
}
template <int L>
static int run_x_kind(int kind, const StArgs& a, dim3 g, cudaStream_t st) {
  switch (kind) {
    case K_DER1: return run_x<L, K_DER1>(a, g, st);
    case K_DER2: return run_x<L, K_DER2>(a, g, st);
    case K_FIL: return run_x<L, K_FIL>(a, g, st);
    case K_DVP: return run_x<L, K_DVP>(a, g, st);
    case K_IVP: return run_x<L, K_IVP>(a, g, st);
    case K_DPV: return run_x<L, K_DPV>(a, g, st);
    case K_IPV: return run_x<L, K_IPV>(a, g, st);
    default: return X3D_ERR_UNSUPPORTED;
  }
}

template <int FC, int KA, int KB, int MODE, bool OUT64>
static int run_yz(const StArgs& a, dim3 g, cudaStream_t st) {
  static bool conf = false;
  constexpr size_t sm = st_smem<FC, MODE == SM_SUM ? 2 : 1>();
  return launch_dyn(stag_yz<FC, KA, KB, MODE, OUT64>, g, dim3(CP, FC), sm, st, a, conf);
}
template <int KA, int KB, int MODE, bool OUT64>
static int run_yz_fc(int FC, const StArgs& a, dim3 g, cudaStream_t st) {
  if (FC == 16) return run_yz<16, KA, KB, MODE, OUT64>(a, g, st);
  if (FC == 32) return run_yz<32, KA, KB, MODE, OUT64>(a, g, st);
  return run_yz<64, KA, KB, MODE, OUT64>(a, g, st);
}

// Line geometry and the circulant coefficients of plans pA (and pB).
static int st_setup(const Ctx* c, OpPlan* pA, OpPlan* pB, const int* dims, StArgs& a, dim3& g, int& L, int& FC) {
  const int axis = pA->axis;
  if (pB && pB->axis != axis) return X3D_ERR_ARG;
  if (!stag_fast_ok(c, axis, dims)) return X3D_ERR_UNSUPPORTED;
  const int n = dims[axis];
  if (pA->nin != n || pA->nout != n || (pB && (pB->nin != n || pB->nout != n))) return X3D_ERR_SHAPE;
  const long long nx = dims[0], ny = dims[1], nz = dims[2];
  if (axis == 0) {
    L = n / 32;
    FC = 32;
    a.na = (int)ny;
    a.sa = nx;
    a.sb = nx * ny;
    a.rs = 1;
    if (nz > 65535) return X3D_ERR_UNSUPPORTED;
    g = dim3((unsigned)((ny + SXW - 1) / SXW), (unsigned)nz);
  } else {
    L = YL;
    FC = n / YL;
    a.na = (int)nx;
    a.sa = 1;
    a.sb = (axis == 1) ? nx * ny : nx;
    a.rs = (int)((axis == 1) ? nx : nx * ny);
    const long long planes = (axis == 1) ? nz : ny;
    if (planes > 65535) return X3D_ERR_UNSUPPORTED;
    g = dim3((unsigned)(nx / (2 * CP)), (unsigned)planes);
  }
  int rc = fill_circ(pA, L, axis == 0 ? 32 : FC - 1, a.A);
  if (rc == X3D_OK && pB) rc = fill_circ(pB, L, axis == 0 ? 32 : FC - 1, a.B);
  return rc;
}

static bool aligned(const void* p, size_t b) { return reinterpret_cast<uintptr_t>(p) % b == 0; }

}  // namespace lk

using namespace lk;

bool stag_fast_ok(const Ctx* c, int axis, const int* dims) {
  const int n = dims[axis];
  if (!c->fast_lines || !c->ax[axis].periodic || (n != 128 && n != 256 && n != 512)) return false;
  if (axis != 0 && dims[0] % (2 * CP) != 0) return false;
  const long long rs = (axis == 0) ? 1 : (axis == 1 ? (long long)dims[0] : (long long)dims[0] * dims[1]);
  return (long long)n * rs < (1LL << 31);
}

int stag_one(Ctx* c, OpPlan* p, float* out, const float* in, const int* dims, cudaStream_t st, float* cor_h,
             float* cor_l) {
  StArgs a;
  std::memset(&a, 0, sizeof(a));
  dim3 g;
  int L = 0, FC = 0;
  int rc = st_setup(c, p, nullptr, dims, a, g, L, FC);
  if (rc != X3D_OK) return rc;
  a.in0 = in;
  a.out0 = out;
  if (cor_h || cor_l) {
    if (p->axis != 0 || !cor_h || !cor_l) return X3D_ERR_UNSUPPORTED;
    if (!aligned(cor_h, 16) || !aligned(cor_l, 16)) return X3D_ERR_UNSUPPORTED;
    a.ch = cor_h;
    a.cl = cor_l;
  }
  if (p->axis == 0) {
    if (!a.ch && !aligned(out, 16)) return X3D_ERR_UNSUPPORTED;
    if (L == 4) return run_x_kind<4>(p->kind, a, g, st);
    if (L == 8) return run_x_kind<8>(p->kind, a, g, st);
    return run_x_kind<16>(p->kind, a, g, st);
  }
  if (!aligned(out, 8) || !aligned(in, 8)) return X3D_ERR_UNSUPPORTED;
  switch (p->kind) {
    case K_DVP: return run_yz_fc<K_DVP, K_DVP, SM_ONE, false>(FC, a, g, st);
    case K_IVP: return run_yz_fc<K_IVP, K_IVP, SM_ONE, false>(FC, a, g, st);
    case K_DPV: return run_yz_fc<K_DPV, K_DPV, SM_ONE, false>(FC, a, g, st);
    case K_IPV: return run_yz_fc<K_IPV, K_IPV, SM_ONE, false>(FC, a, g, st);
    default: return X3D_ERR_UNSUPPORTED;
  }
}

int stag_sum(Ctx* c, OpPlan* pA, const float* inA, OpPlan* pB, const float* inB, void* out, bool out64,
             const int* dims, cudaStream_t st) {
  if (pA->axis == 0) return X3D_ERR_UNSUPPORTED;
  StArgs a;
  std::memset(&a, 0, sizeof(a));
  dim3 g;
  int L = 0, FC = 0;
  int rc = st_setup(c, pA, pB, dims, a, g, L, FC);
  if (rc != X3D_OK) return rc;
  if (!aligned(out, out64 ? 16 : 8) || !aligned(inA, 8) || !aligned(inB, 8)) return X3D_ERR_UNSUPPORTED;
  a.in0 = inA;
  a.in1 = inB;
  a.out0 = out;
  if (pA->kind == K_DVP && pB->kind == K_IVP && !out64) return run_yz_fc<K_DVP, K_IVP, SM_SUM, false>(FC, a, g, st);
  if (pA->kind == K_IVP && pB->kind == K_DVP && out64) return run_yz_fc<K_IVP, K_DVP, SM_SUM, true>(FC, a, g, st);
  if (pA->kind == K_IVP && pB->kind == K_DVP && !out64) return run_yz_fc<K_IVP, K_DVP, SM_SUM, false>(FC, a, g, st);
  return X3D_ERR_UNSUPPORTED;
}

int stag_dual(Ctx* c, OpPlan* pA, float* outA, OpPlan* pB, float* outB, const float* in, const int* dims,
              cudaStream_t st) {
  if (pA->axis == 0) return X3D_ERR_UNSUPPORTED;
  StArgs a;
  std::memset(&a, 0, sizeof(a));
  dim3 g;
  int L = 0, FC = 0;
  int rc = st_setup(c, pA, pB, dims, a, g, L, FC);
  if (rc != X3D_OK) return rc;
  if (!aligned(outA, 8) || !aligned(outB, 8) || !aligned(in, 8)) return X3D_ERR_UNSUPPORTED;
  a.in0 = in;
  a.out0 = outA;
  a.out1 = outB;
  if (pA->kind == K_IPV && pB->kind == K_DPV) return run_yz_fc<K_IPV, K_DPV, SM_DUAL, false>(FC, a, g, st);
  return X3D_ERR_UNSUPPORTED;
}

}  // namespace x3d
