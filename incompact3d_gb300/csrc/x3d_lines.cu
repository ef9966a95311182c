// Host launcher of the generic compact-operator line kernel
// (x3d_line_kernel.cuh): per-operator plan finalisation (chunk fix-up
// factors, device upload) and argument marshalling.
#include <type_traits>

#include <cmath>
#include <cstdint>

#include "x3d_line_fast.cuh"

namespace x3d {

using namespace lk;

namespace lk {
// Fast-path coefficients of a (periodic, FP32) plan.
void fill_fast_op(const OpPlan* p, FastOp<float>& a) {
  const int n = p->nout;
  const int L = n / FCHUNKS;
  const float* dv = p->dev32;
  a.s = dv; a.f = dv + n; a.w = dv + 2 * n; a.pf = dv + 3 * n; a.qb = dv + 4 * n; a.rsm = dv + 5 * n;
  a.ca = (float)p->ca; a.cb = (float)p->cb; a.cc = (float)p->cc; a.cd = (float)p->cd;
  a.alpha = (float)p->alpha;
  a.den = (float)p->den;
  a.nterms_int = 4;
  if (p->kind == K_DER2 && p->cc == 0.0 && p->cd == 0.0) a.nterms_int = 2;
  if ((p->kind == K_IVP || p->kind == K_IPV) && p->cd == 0.0) a.nterms_int = 3;
  const int mid = n / 2;
  a.s_inf = (float)p->s[mid];
  a.f_inf = (float)p->f[mid];
  a.w_inf = (float)p->w[mid];
  a.g_inf = (float)(-(p->f[mid] * p->w[mid]));
  for (int c = 0; c < FCHUNKS; ++c) {
    const int s0 = c * L, e0 = s0 + L - 1;
    a.pfe[c] = (float)p->pf[e0];
    a.qbs[c] = (float)p->qb[s0];
    bool uni = true, sm = false;
    for (int r = s0; r <= e0; ++r) {
      uni = uni && (float)p->s[r] == a.s_inf && (float)p->f[r] == a.f_inf && (float)p->w[r] == a.w_inf;
      sm = sm || (float)p->rsm[r] != 0.0f;
    }
    a.mode[c] = (uni ? 1 : 0) | (sm ? 2 : 0);
  }
  // fix-up factors of uniform chunks, by the same running products in binary32
  const float m = -a.s_inf;
  float P = m;
  for (int k = 0; k < 32; ++k) {
    a.pw[k] = (k < L) ? P : 0.f;
    P = P * m;
  }
  float Q = a.g_inf;
  for (int k = L - 1; k >= 0; --k) {
    a.qw[k] = Q;
    Q = Q * a.g_inf;
  }
  for (int k = L; k < 32; ++k) a.qw[k] = 0.f;
}

// Line geometry of an axis for the fast kernels: lines (a, b), row stride.
void fast_geometry(int axis, int n, const int* dims_in, long long* sa, long long* sb, long long* rs, int* na,
                   dim3* grid) {
  const long long nx = dims_in[0], ny = dims_in[1], nz = dims_in[2];
  if (axis == 0) {
    *na = (int)ny; *sa = n; *sb = ny * n; *rs = 1;
    *grid = dim3((unsigned)((ny + LANES - 1) / LANES), (unsigned)nz);
  } else if (axis == 1) {
    *na = (int)nx; *sa = 1; *sb = nx * n; *rs = nx;
    *grid = dim3((unsigned)((nx + LANES - 1) / LANES), (unsigned)nz);
  } else {
    *na = (int)nx; *sa = 1; *sb = nx; *rs = nx * ny;
    *grid = dim3((unsigned)((nx + LANES - 1) / LANES), (unsigned)ny);
  }
}

}  // namespace lk

namespace {

template <typename T>
int dispatch(const LineArgs<T>& a, int kind, bool xl, int lmax, dim3 grid, size_t smem, cudaStream_t st) {
  switch (kind) {
    case K_DER1: return line_dispatch<K_DER1>(a, xl, lmax, grid, smem, st);
    case K_DER2: return line_dispatch<K_DER2>(a, xl, lmax, grid, smem, st);
    case K_FIL: return line_dispatch<K_FIL>(a, xl, lmax, grid, smem, st);
    case K_DVP: return line_dispatch<K_DVP>(a, xl, lmax, grid, smem, st);
    case K_IVP: return line_dispatch<K_IVP>(a, xl, lmax, grid, smem, st);
    case K_DPV: return line_dispatch<K_DPV>(a, xl, lmax, grid, smem, st);
    case K_IPV: return line_dispatch<K_IPV>(a, xl, lmax, grid, smem, st);
  }
  return X3D_ERR_ARG;
}

int fdispatch(const FastArgs<float>& a, int kind, bool xl, int L, dim3 grid, size_t smem, cudaStream_t st) {
  switch (kind) {
    case K_DER1: return fast_dispatch<K_DER1>(a, xl, L, grid, smem, st);
    case K_DER2: return fast_dispatch<K_DER2>(a, xl, L, grid, smem, st);
    case K_FIL: return fast_dispatch<K_FIL>(a, xl, L, grid, smem, st);
    case K_DVP: return fast_dispatch<K_DVP>(a, xl, L, grid, smem, st);
    case K_IVP: return fast_dispatch<K_IVP>(a, xl, L, grid, smem, st);
    case K_DPV: return fast_dispatch<K_DPV>(a, xl, L, grid, smem, st);
    case K_IPV: return fast_dispatch<K_IPV>(a, xl, L, grid, smem, st);
  }
  return X3D_ERR_ARG;
}

// Periodic lines of 16*L points (L = 8, 16, 32) in FP32 take the fast path.
int launch_fast(OpPlan* p, float* out, const float* in, const int* dims_in, cudaStream_t st,
                const Fuse<float>* fz) {
  const int n = p->nout;
  const int L = n / FCHUNKS;
  FastArgs<float> a;
  std::memset(&a, 0, sizeof(a));
  a.in = in;
  a.out = out;
  a.n = n;
  dim3 grid;
  const bool xl = (p->axis == 0);
  fast_geometry(p->axis, n, dims_in, &a.sa, &a.sb, &a.rs, &a.na, &grid);
  if (grid.y > 65535) return X3D_ERR_UNSUPPORTED;
  fill_fast_op(p, a.op);
  if (fz) a.fz = *fz;
  const size_t smem = fast_smem<float>(n, xl);
  return fdispatch(a, p->kind, xl, L, grid, smem, st);
}

template <typename T>
const T* plan_dev(const OpPlan* p);
template <>
const double* plan_dev<double>(const OpPlan* p) { return p->dev64; }
template <>
const float* plan_dev<float>(const OpPlan* p) { return p->dev32; }

}  // namespace

// Chunk length and fix-up factors for a plan (host only).
int finalize_plan(OpPlan* p) {
  const int n = p->nout;
  const int L = (n + CHUNKS - 1) / CHUNKS;
  if (L > 32) return X3D_ERR_UNSUPPORTED;  // lines longer than 512 points
  p->L = L;
  p->pf.assign(n, 0.0);
  p->qb.assign(n, 0.0);
  for (int c = 0; c * L < n; ++c) {
    const int s0 = c * L, e0 = std::min(s0 + L, n) - 1;
    double acc = 1.0;
    for (int r = s0; r <= e0; ++r) {
      acc = acc * (-p->s[r]);
      p->pf[r] = acc;
    }
    acc = 1.0;
    for (int r = e0; r >= s0; --r) {
      acc = acc * (-(p->f[r] * p->w[r]));
      p->qb[r] = acc;
    }
  }
  return X3D_OK;
}

// Device copies of a plan's vectors, made on first launch.
int upload_plan(OpPlan* p) {
  if (p->dev64) return X3D_OK;
  const int n = p->nout;
  std::vector<double> h64(6 * (size_t)n);
  std::vector<float> h32(6 * (size_t)n);
  const dvec* parts[6] = {&p->s, &p->f, &p->w, &p->pf, &p->qb, &p->rsm};
  for (int q = 0; q < 6; ++q)
    for (int r = 0; r < n; ++r) {
      h64[(size_t)q * n + r] = (*parts[q])[r];
      h32[(size_t)q * n + r] = (float)(*parts[q])[r];
    }
  double* d64 = nullptr;
  float* d32 = nullptr;
  if (cudaMalloc(&d64, h64.size() * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
  if (cudaMalloc(&d32, h32.size() * sizeof(float)) != cudaSuccess) {
    cudaFree(d64);
    return X3D_ERR_NOMEM;
  }
  cudaError_t e = cudaMemcpy(d64, h64.data(), h64.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d32, h32.data(), h32.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d64);
    cudaFree(d32);
    return cuda_status(e);
  }
  p->dev64 = d64;
  p->dev32 = d32;
  return X3D_OK;
}

template <typename T>
int launch_line_op(Ctx* c, OpPlan* p, T* out, const T* in, const int* dims_in, const T* pp, cudaStream_t st,
                   const Fuse<T>* fz) {
  if (!out || !in) return X3D_ERR_ARG;
  if (dims_in[p->axis] != p->nin) return X3D_ERR_SHAPE;
  const int up = upload_plan(p);
  if (up != X3D_OK) return up;
  // binary32 periodic x lines without a fused load / store: one warp per line
  // in circulant form (x3d_stag_circ.cu)
  if (std::is_same<T, float>::value && p->axis == 0 && p->periodic && p->nin == p->nout && pp == nullptr &&
      (fz == nullptr || (fz->in2 == nullptr && !fz->active)) && stag_fast_ok(c, 0, dims_in) &&
      reinterpret_cast<uintptr_t>(out) % 16 == 0) {
    const int rc = stag_one(c, p, (float*)out, (const float*)in, dims_in, st);
    if (rc != X3D_ERR_UNSUPPORTED) return rc;
  }
  if (std::is_same<T, float>::value && p->periodic && p->nin == p->nout && pp == nullptr && c->fast_lines &&
      p->nout % FCHUNKS == 0 && (p->nout / FCHUNKS == 8 || p->nout / FCHUNKS == 16 || p->nout / FCHUNKS == 32))
    return launch_fast(p, (float*)out, (const float*)in, dims_in, st, (const Fuse<float>*)fz);
  LineArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.in = in;
  a.out = out;
  a.nin = p->nin;
  a.nout = p->nout;
  a.L = p->L;
  const long long nx = dims_in[0], ny = dims_in[1], nz = dims_in[2];
  dim3 grid;
  const bool xl = (p->axis == 0);
  if (p->axis == 0) {
    a.na = (int)ny;
    a.sa_in = p->nin; a.sb_in = ny * p->nin; a.rs_in = 1;
    a.sa_out = p->nout; a.sb_out = ny * p->nout; a.rs_out = 1;
    grid = dim3((unsigned)((ny + LANES - 1) / LANES), (unsigned)nz);
  } else if (p->axis == 1) {
    a.na = (int)nx;
    a.sa_in = 1; a.sb_in = nx * p->nin; a.rs_in = nx;
    a.sa_out = 1; a.sb_out = nx * p->nout; a.rs_out = nx;
    grid = dim3((unsigned)((nx + LANES - 1) / LANES), (unsigned)nz);
  } else {
    a.na = (int)nx;
    a.sa_in = 1; a.sb_in = nx; a.rs_in = nx * ny;
    a.sa_out = 1; a.sb_out = nx; a.rs_out = nx * ny;
    grid = dim3((unsigned)((nx + LANES - 1) / LANES), (unsigned)ny);
  }
  if (grid.y > 65535) return X3D_ERR_UNSUPPORTED;
  const T* dv = plan_dev<T>(p);
  const int n = p->nout;
  a.s = dv; a.f = dv + n; a.w = dv + 2 * n; a.pf = dv + 3 * n; a.qb = dv + 4 * n; a.rsm = dv + 5 * n;
  a.pp = pp;
  a.ca = (T)p->ca; a.cb = (T)p->cb; a.cc = (T)p->cc; a.cd = (T)p->cd;
  a.alpha = (T)p->alpha;
  a.den = (T)p->den;
  a.periodic = p->periodic ? 1 : 0;
  a.nterms_int = 4;
  if (p->kind == K_DER2 && p->cc == 0.0 && p->cd == 0.0) a.nterms_int = 2;
  if ((p->kind == K_IVP || p->kind == K_IPV) && p->cd == 0.0) a.nterms_int = 3;
  a.nbrows = p->nbrows;
  for (int q = 0; q < p->nbrows; ++q) {
    const BRow& s = p->brows[q];
    BRowD<T>& d = a.brows[q];
    d.row = (short)s.row;
    d.nterms = (signed char)s.nterms;
    for (int t = 0; t < kMaxTerms; ++t) {
      d.coef[t] = (T)s.coef[t];
      d.nent[t] = (signed char)s.nent[t];
      for (int e = 0; e < kMaxEnt; ++e) {
        d.idx[t][e] = (short)s.idx[t][e];
        d.mult[t][e] = (signed char)s.mult[t][e];
      }
    }
  }
  if (fz) a.fz = *fz;
  // circulant form of periodic lines whose chunks are all full: two
  // recurrences with a constant coefficient and cyclic chunk carries instead
  // of the Thomas sweeps with per-row factors and the Sherman-Morrison pass
  // (two fewer operations per point on the FP64-bound path); carries whose
  // weight falls below the precision's resolution (2^-60 binary64, 2^-32
  // binary32) are dropped
  if (p->periodic && p->nin == p->nout && p->nout == CHUNKS * p->L && p->L <= 32 && plan_is_circulant(p)) {
    const double al = p->alpha;
    const double mu = 2.0 * al / (1.0 + std::sqrt(1.0 - 4.0 * al * al));
    const double sc = 1.0 + mu * mu;
    const double A = std::pow(-mu, p->L);
    const double lim = std::is_same<T, double>::value ? std::ldexp(1.0, -60) : std::ldexp(1.0, -32);
    int J = 1;
    for (double w = std::fabs(A); J < CHUNKS - 1 && w >= lim; w *= std::fabs(A)) ++J;
    if (std::pow(std::fabs(A), J) < lim) {
      a.circ = 1;
      a.cJ = J;
      a.cnmu = (T)(-mu);
      a.cA = (T)A;
      a.ca = (T)(p->ca * sc); a.cb = (T)(p->cb * sc); a.cc = (T)(p->cc * sc); a.cd = (T)(p->cd * sc);
      for (int k = 0; k < p->L; ++k) {
        a.cpw[k] = (T)std::pow(-mu, k + 1);
        a.cqw[k] = (T)std::pow(-mu, p->L - k);
      }
    }
  }
  const int lmax = (p->L <= 8) ? 8 : (p->L <= 16) ? 16 : 32;
  const size_t smem = line_smem<T>(p->nin, p->nout);
  if (smem > 227 * 1024) return X3D_ERR_UNSUPPORTED;
  return dispatch<T>(a, p->kind, xl, lmax, grid, smem, st);
}

// Host copy of a plan (diagnostics / CPU emulation of the kernel).
int plan_info(Ctx* c, int axis, int kind, int npaire, int coefset, double* sc, double* vecs, double* brows) {
  OpPlan* p = nullptr;
  const int rc = get_plan(c, axis, kind, npaire, coefset, &p);
  if (rc != X3D_OK) return rc;
  const int n = p->nout;
  int nt = 4;
  if (p->kind == K_DER2 && p->cc == 0.0 && p->cd == 0.0) nt = 2;
  if ((p->kind == K_IVP || p->kind == K_IPV) && p->cd == 0.0) nt = 3;
  const double v[16] = {(double)p->nin, (double)n, (double)p->L, p->periodic ? 1.0 : 0.0, p->ca, p->cb, p->cc,
                        p->cd, p->alpha, p->den, (double)p->nbrows, (double)nt, (double)CHUNKS,
                        (p->periodic && plan_is_circulant(p)) ? 1.0 : 0.0, 0, 0};
  if (sc) std::memcpy(sc, v, sizeof(v));
  const dvec* parts[6] = {&p->s, &p->f, &p->w, &p->pf, &p->qb, &p->rsm};
  if (vecs)
    for (int q = 0; q < 6; ++q) std::memcpy(vecs + (size_t)q * n, parts[q]->data(), n * sizeof(double));
  if (brows)
    for (int q = 0; q < p->nbrows; ++q) {
      const BRow& b = p->brows[q];
      double* o = brows + q * (2 + kMaxTerms * (2 + 2 * kMaxEnt));
      o[0] = b.row;
      o[1] = b.nterms;
      for (int t = 0; t < kMaxTerms; ++t) {
        double* ot = o + 2 + t * (2 + 2 * kMaxEnt);
        ot[0] = b.coef[t];
        ot[1] = b.nent[t];
        for (int e = 0; e < kMaxEnt; ++e) {
          ot[2 + 2 * e] = b.idx[t][e];
          ot[3 + 2 * e] = b.mult[t][e];
        }
      }
    }
  return n;
}

template int launch_line_op<double>(Ctx*, OpPlan*, double*, const double*, const int*, const double*, cudaStream_t,
                                   const Fuse<double>*);
template int launch_line_op<float>(Ctx*, OpPlan*, float*, const float*, const int*, const float*, cudaStream_t,
                                  const Fuse<float>*);

}  // namespace x3d
