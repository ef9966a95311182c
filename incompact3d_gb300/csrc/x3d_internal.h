// Internal declarations shared by the libx3dgpu translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "x3d_gpu.h"

namespace x3d {

typedef std::vector<double> dvec;

// Operator kinds: one generic "banded right-hand side + tridiagonal solve
// (+ periodic Sherman-Morrison)" kernel covers all of them.
enum OpKind { K_DER1 = 0, K_DER2 = 1, K_FIL = 2, K_DVP = 3, K_IVP = 4, K_DPV = 5, K_IPV = 6, K_COUNT = 7 };

constexpr int kMaxTerms = 6;   // terms in one boundary-row expression
constexpr int kMaxEnt = 4;     // signed samples inside one term
constexpr int kMaxBRows = 10;  // boundary rows per operator (both ends)

// One boundary row:  t[row] = sum_t coef[t] * (sum_e mult[t][e] * u[idx[t][e]])
// evaluated left to right, exactly the way the reference writes the row.
struct BRow {
  int row = 0;
  int nterms = 0;
  double coef[kMaxTerms] = {0};
  int nent[kMaxTerms] = {0};
  int idx[kMaxTerms][kMaxEnt] = {{0}};
  int mult[kMaxTerms][kMaxEnt] = {{0}};
};

// Per-axis coefficients: the restatement of the reference's init-time
// coefficient computation (src/schemes.f90, src/filters.f90).
struct AxisCoef {
  int n = 0, nm = 0, ncl1 = 0, ncln = 0;
  bool periodic = true;
  double len = 0, d = 0, d2 = 0;
  // first derivative
  double alfai, afi, bfi, af1, bf1, cf1, af2, afm, afn, bfn, cfn, alfa1, alfa2, alfam, alfan;
  // second derivative
  double alsai, asi, bsi, csi, dsi, as1, bs1, cs1, ds1, as2, as3, bs3, as4, bs4, cs4, asn, bsn, csn, dsn, asm_,
      ast, bst, astt, bstt, cstt;
  // staggered
  double alcai6, aci6, bci6, ailcai6, aici6, bici6, cici6s, dici6;
  // filter
  double fiali, fiai, fibi, fici, fidi, fia2, fib2, fic2, fid2, fia3, fib3, fic3, fid3, fie3, fif3, fiam, fibm,
      ficm, fidm, fiap, fibp, ficp, fidp, fiep, fifp;
  // coefficient vectors, indexed by X3D_COEF_*
  dvec vecs[X3D_COEF_COUNT];
};

// Plan of one operator (axis, kind, npaire, coefficient set): everything the
// generic line kernel needs, on host and in device memory.
struct OpPlan {
  int axis = 0, kind = 0, npaire = 0, coefset = 0;
  int nin = 0, nout = 0;
  bool periodic = false;
  double ca = 0, cb = 0, cc = 0, cd = 0;  // interior stencil coefficients
  double alpha = 0, den = 1;              // Sherman-Morrison
  int nbrows = 0;
  BRow brows[kMaxBRows];
  dvec s, f, w, rsm;  // Thomas factors and the precomputed SM vector
  int L = 0;          // chunk length the fix-up factors below were built for
  dvec pf, qb;        // chunked-solve fix-up factors
  // device copies: [s | f | w | pf | qb | rsm] x nout, in f64 and f32
  double* dev64 = nullptr;
  float* dev32 = nullptr;
};

struct Ctx;

// Build all per-axis coefficients (host).  Returns X3D_OK or an error.
int build_axis(AxisCoef& a, int n, double len, int ncl1, int ncln, const x3d_numopts& o);
// Build the plan of one operator (host part).  Returns X3D_OK or an error.
int build_plan(const AxisCoef& a, int axis, int kind, int npaire, int coefset, OpPlan& p);
// True when a periodic plan's Thomas factors are those of the corner-modified
// circulant [alpha, 1, alpha] (the solve is then A^-1 b, A circulant).
bool plan_is_circulant(const OpPlan* p);
// Default coefficient set for (kind, npaire) as the reference's callers pick it.
int default_coefset(int kind, int npaire);
// Index (X3D_COEF_*) of the (f, s, w) vectors of a plan's coefficient set.
void coef_indices(const AxisCoef& a, int kind, int coefset, int* fi, int* si, int* wi);

// Poisson tables (periodic): modified wavenumber^2 and interpolation transfer.
void waves_tables(const AxisCoef& a, dvec& k2, dvec& tr);
// poisson_11x: kxyz (re, im) per spectral point (i, j, k < NZ/2+1), x and y
// free-slip, z free-slip or periodic (x3d_plan.cpp).
void kxyz_11x(const AxisCoef& ax, const AxisCoef& ay, const AxisCoef& az, dvec& kre, dvec& kim);

// Mesh stretching in y and its device copies.
struct Stretch {
  int istret = 0;
  double beta = 0, alpha = 0;
  dvec yp, ypi, ppy, pp2y, pp4y, ppyi, pp2yi, pp4yi;
  double* d_ppy = nullptr;  // device: ppy | pp2y | pp4y | ppyi (ny each)
};
// Stretching metrics (src/stretching.f90) or the uniform defaults.
int build_stretch(const x3d_grid& g, const AxisCoef& ay, Stretch& st);
// poisson_010 tables of a non-periodic y axis: yky, yk2 (ny entries), the
// transfer function (nym) and the shift factors sin/cos((j-1) pi/(2 nym)).
void waves_y010(const AxisCoef& a, int istret, double yly, dvec& yky, dvec& yk2, dvec& tr, dvec& sa, dvec& sb);

// Device scratch owned by a context, grown on demand (used by the stand-alone
// projection entry points, which have no solver to borrow work fields from).
struct Workspace {
  void* buf = nullptr;
  size_t bytes = 0;
  ~Workspace() {
    if (buf) cudaFree(buf);
  }
};

struct Ctx {
  x3d_grid grid;
  x3d_numopts opts;
  int device = 0;
  int num_sms = 0;
  bool fast_lines = true;  // FP32 periodic lines of 16*L points use line_fast
  AxisCoef ax[3];
  std::map<int, std::unique_ptr<OpPlan>> plans;  // key = packed (axis,kind,npaire,coefset)
  // Poisson device tables
  double* d_k2[3] = {nullptr, nullptr, nullptr};
  double* d_tr[3] = {nullptr, nullptr, nullptr};
  double* d_twid = nullptr;  // FFT twiddles (see x3d_fft.cu)
  float* d_twid32 = nullptr;
  float* d_twid_df = nullptr;             // twiddles as binary32 hi/lo pairs
  float2* d_k2df[3] = {nullptr, nullptr, nullptr};  // k2 / transfer tables as hi/lo pairs
  float2* d_trdf[3] = {nullptr, nullptr, nullptr};
  int twid_n = 0;
  void* d_inv[3] = {nullptr, nullptr, nullptr};  // poisson_000 factor tables: f64, f32, hi/lo f32
  void* fft_work = nullptr;  // complex spectrum buffer
  size_t fft_work_bytes = 0;
  Stretch st;
  double* d_p010 = nullptr;  // poisson_010 tables (see x3d_fft.cu)
  double* d_p11 = nullptr;   // poisson_11x tables (see x3d_fft.cu)
  double p010_xa[2] = {0, 0};  // stretching constants xa0, xa1 of matrice_refinement
  std::unique_ptr<Workspace> ws;
  ~Ctx();
};

// Device copies of ppy | pp2y | pp4y | ppyi (uploaded on first use).
int stretch_device(Ctx* c, const double** out);
// poisson_010 (x, z periodic; y non-periodic, stretched or not), FP64.
int poisson_010(Ctx* c, double* rhs, cudaStream_t st);
// poisson_11x (src/poisson.f90:1019-1465): x and y free-slip, z free-slip or
// periodic, uniform mesh, FP64 (x3d_fft.cu).
int poisson_11x(Ctx* c, double* rhs, cudaStream_t st);
// poisson_000 in double-float arithmetic on a binary32 right-hand side,
// solution rounded once to binary32 in place (the mixed-precision step).
int poisson_periodic_f32io(Ctx* c, float* p, cudaStream_t st);
bool is_11x(const Ctx* c);

// Device scratch of at least `bytes` bytes (contents undefined).
int ctx_workspace(Ctx* c, size_t bytes, void** out);

// Learned SGS closure (x3d_mlp.cu): tau_ij from the 9 gradient fields and the
// filter width.
struct Mlp;
int mlp_les_tau(Mlp* m, const double* const* g9, double delta, double* const* tau6, long long n, int num_sms,
                cudaStream_t st);

// Shape of the closure and offsets of its parameter array:
// W1[64][10], b1[64], W2[64][64], b2[64], W3[6][64], b3[6].
namespace mlpdim {
constexpr int NI = 10, NH = 64, NO = 6;
constexpr int OW1 = 0;
constexpr int OB1 = OW1 + NH * NI;
constexpr int OW2 = OB1 + NH;
constexpr int OB2 = OW2 + NH * NH;
constexpr int OW3 = OB2 + NH;
constexpr int OB3 = OW3 + NO * NH;
constexpr int NPAR = OB3 + NO;  // 5254
}  // namespace mlpdim

// Tensor-core (tcgen05) inference of the closure (x3d_mlp_tc.cu).  The weights
// are packed once per parameter change into the BF16 hi / lo image the MMAs
// read (MLP_TC_WP_BYTES, 16-byte aligned); err (device int) is set to 1 when a
// bounded wait on the tensor core or the weight copy runs out.  Features come
// from X[n][10] (FP32 rows) when X is non-null, else from the 9 gradient
// fields g9 and delta; results go to Y[n][6] or to tau6.
constexpr int MLP_TC_WP_BYTES = 24576;
int mlp_tc_pack(const float* P, void* wp, cudaStream_t st);
int mlp_tc_infer(const float* P, const float* sc, const void* wp, int* err, const float* X, float* Y,
                 const double* const* g9, float delta, double* const* tau6, long long n, int num_sms,
                 cudaStream_t st);

// Device copies of a plan's vectors (made on first use).
int upload_plan(OpPlan* p);
// Fused momentum right-hand side along one axis, binary32 periodic lines in
// circulant form (x3d_conv_diff.cu): out = nu*C(uq) + a1 - (A(ua*uq) + ua*B(uq))/2
// with A, B first-derivative and C second-derivative plans of that axis; a1
// may be null or alias out.  X3D_ERR_UNSUPPORTED where no kernel applies
// (rhs_axis_fast_ok false).
int rhs_axis_fast(Ctx* c, OpPlan* pA, OpPlan* pB, OpPlan* pC, float* out, const float* ua, const float* uq,
                  const float* a1, float nu, const int* dims, cudaStream_t st);
bool rhs_axis_fast_ok(const Ctx* c, int axis, const int* dims);
// Staggered operators of binary32 periodic lines in circulant form
// (x3d_stag_circ.cu): one solve (x, y, z), the sum of two solves on two
// inputs (y/z: deryvp + interyvp, interzvp + derzvp with FP64 output) and two
// solves of one input (y/z: interzpv + derzpv, interypv + derypv).
// X3D_ERR_UNSUPPORTED where stag_fast_ok is false or the pair is not one of
// those.
bool stag_fast_ok(const Ctx* c, int axis, const int* dims);
// cor_h / cor_l (x lines only): instead of writing out, subtract the result
// from the double-float pair (cor_h, cor_l), the fused cor_vel of the step.
int stag_one(Ctx* c, OpPlan* p, float* out, const float* in, const int* dims, cudaStream_t st,
             float* cor_h = nullptr, float* cor_l = nullptr);
int stag_sum(Ctx* c, OpPlan* pA, const float* inA, OpPlan* pB, const float* inB, void* out, bool out64,
             const int* dims, cudaStream_t st);
int stag_dual(Ctx* c, OpPlan* pA, float* outA, OpPlan* pB, float* outB, const float* in, const int* dims,
              cudaStream_t st);

// Get (building on first use) the device plan of an operator.
int get_plan(Ctx* c, int axis, int kind, int npaire, int coefset, OpPlan** out);

// Optional fusion of the pointwise work around a compact operator:
//   input  u = in * in2                       (in2 != null)
//   output o = cr*t + c1*a1 + c2*a2 + y*t     (active != 0; null operands skipped)
// a1, a2, y have the output's layout; the output may alias a1 or a2.
template <typename T>
struct Fuse {
  const T* in2 = nullptr;
  const T* a1 = nullptr;
  const T* a2 = nullptr;
  const T* y = nullptr;
  T cr = T(1), c1 = T(0), c2 = T(0);
  int active = 0;
};

// Launch the compact-operator line kernel (generic or fast path).  T = double
// or float; fz may be null.
template <typename T>
int launch_line_op(Ctx* c, OpPlan* p, T* out, const T* in, const int* dims_in, const T* pp, cudaStream_t st,
                   const Fuse<T>* fz = nullptr);

// Host copy of a plan: sc[16] scalars, vecs[6*nout] = s,f,w,pf,qb,rsm,
// brows[kMaxBRows*(2+kMaxTerms*(2+2*kMaxEnt))].  Returns nout or an error.
int plan_info(Ctx* c, int axis, int kind, int npaire, int coefset, double* sc, double* vecs, double* brows);

// Poisson (periodic, all three directions).  precision 0: FP64 FFT, 1: FP32 FFT.
int poisson_periodic(Ctx* c, double* rhs, int precision, cudaStream_t st);
// Same solve with all scratch in a fixed device array (no allocation).
int poisson_periodic_noalloc(Ctx* c, double* rhs, cudaStream_t st);

// Records the CUDA error behind an X3D_ERR_CUDA (see x3d_last_cuda_error).
void note_cuda_error(cudaError_t e);
inline int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return X3D_OK;
  note_cuda_error(e);
  return X3D_ERR_CUDA;
}

}  // namespace x3d
