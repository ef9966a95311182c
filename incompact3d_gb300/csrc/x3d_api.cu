// C ABI of libx3dgpu.so: context management and the per-routine entry points
// that mirror the reference's Fortran interfaces (see include/x3d_gpu.h).
#include <cstring>

#include "x3d_internal.h"

namespace x3d {

int finalize_plan(OpPlan* p);

Ctx::~Ctx() {
  for (auto& kv : plans) {
    if (kv.second->dev64) cudaFree(kv.second->dev64);
    if (kv.second->dev32) cudaFree(kv.second->dev32);
  }
  for (int a = 0; a < 3; ++a) {
    if (d_k2[a]) cudaFree(d_k2[a]);
    if (d_tr[a]) cudaFree(d_tr[a]);
    if (d_k2df[a]) cudaFree(d_k2df[a]);
    if (d_trdf[a]) cudaFree(d_trdf[a]);
  }
  if (st.d_ppy) cudaFree(st.d_ppy);
  if (d_p010) cudaFree(d_p010);
  if (d_p11) cudaFree(d_p11);
  for (void* t : d_inv)
    if (t) cudaFree(t);
  if (d_twid) cudaFree(d_twid);
  if (d_twid32) cudaFree(d_twid32);
  if (d_twid_df) cudaFree(d_twid_df);
  if (fft_work) cudaFree(fft_work);
}

static thread_local cudaError_t g_last_cuda = cudaSuccess;
void note_cuda_error(cudaError_t e) { g_last_cuda = e; }

int ctx_workspace(Ctx* c, size_t bytes, void** out) {
  if (!c->ws) c->ws.reset(new Workspace());
  Workspace* w = c->ws.get();
  if (w->bytes < bytes) {
    if (w->buf) cudaFree(w->buf);
    w->buf = nullptr;
    w->bytes = 0;
    if (cudaMalloc(&w->buf, bytes) != cudaSuccess) return X3D_ERR_NOMEM;
    w->bytes = bytes;
  }
  *out = w->buf;
  return X3D_OK;
}

int get_plan(Ctx* c, int axis, int kind, int npaire, int coefset, OpPlan** out) {
  if (axis < 0 || axis > 2 || kind < 0 || kind >= K_COUNT) return X3D_ERR_ARG;
  const int key = ((axis * 8 + kind) * 2 + npaire) * 2 + coefset;
  auto it = c->plans.find(key);
  if (it != c->plans.end()) {
    *out = it->second.get();
    return X3D_OK;
  }
  std::unique_ptr<OpPlan> p(new OpPlan());
  int rc = build_plan(c->ax[axis], axis, kind, npaire, coefset, *p);
  if (rc != X3D_OK) return rc;
  rc = finalize_plan(p.get());
  if (rc != X3D_OK) return rc;
  *out = p.get();
  c->plans[key] = std::move(p);
  return X3D_OK;
}

// Device copies of the stretching metrics: ppy | pp2y | pp4y | ppyi.
int stretch_device(Ctx* c, const double** out) {
  if (!c->st.d_ppy) {
    const int ny = c->grid.ny;
    dvec h;
    for (const dvec* v : {&c->st.ppy, &c->st.pp2y, &c->st.pp4y, &c->st.ppyi}) h.insert(h.end(), v->begin(), v->end());
    double* d = nullptr;
    if (cudaMalloc(&d, h.size() * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
    cudaError_t e = cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d);
      return cuda_status(e);
    }
    c->st.d_ppy = d;
    (void)ny;
  }
  *out = c->st.d_ppy;
  return X3D_OK;
}

}  // namespace x3d

using namespace x3d;

namespace {

Ctx* C(x3d_ctx* h) { return reinterpret_cast<Ctx*>(h); }

// Resolve the coefficient set a Fortran caller passed (host vectors) against
// the context's sets.  f/s/w may all be NULL (default set for the parity).
int resolve_set(Ctx* c, int axis, int kind, int npaire, const double* f, const double* s, const double* w,
                int* coefset) {
  if (!f && !s && !w) {
    *coefset = default_coefset(kind, npaire);
    return X3D_OK;
  }
  if (!f || !s || !w) return X3D_ERR_ARG;
  const AxisCoef& a = c->ax[axis];
  for (int cs = 0; cs < 2; ++cs) {
    int fi, si, wi;
    coef_indices(a, kind, cs, &fi, &si, &wi);
    const size_t n = a.vecs[fi].size() * sizeof(double);
    if (std::memcmp(f, a.vecs[fi].data(), n) == 0 && std::memcmp(s, a.vecs[si].data(), n) == 0 &&
        std::memcmp(w, a.vecs[wi].data(), n) == 0) {
      *coefset = cs;
      return X3D_OK;
    }
  }
  return X3D_ERR_COEF;
}

template <typename T>
int run_op(x3d_ctx* h, int axis, int kind, int npaire, int coefset, T* t, const T* u, const int* dims, void* st,
           const T* pp = nullptr) {
  if (!h || !t || !u) return X3D_ERR_ARG;
  if (npaire != 0 && npaire != 1) return X3D_ERR_ARG;
  Ctx* c = C(h);
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return X3D_ERR_SHAPE;
  // dims must be the grid's, except along the operator axis where the
  // staggered pressure-mesh length nm is also accepted on the other axes.
  for (int a = 0; a < 3; ++a)
    if (dims[a] != c->ax[a].n && dims[a] != c->ax[a].nm) return X3D_ERR_SHAPE;
  OpPlan* p = nullptr;
  int rc = get_plan(c, axis, kind, npaire, coefset, &p);
  if (rc != X3D_OK) return rc;
  return launch_line_op<T>(c, p, t, u, dims, pp, (cudaStream_t)st);
}

// The y-metric a y operator multiplies by on a stretched mesh
// (src/derive.f90:409-418 and likewise): `which` 0 = ppy, 3 = ppyi, applied
// only when istret != 0.  A vector passed by the caller must equal the
// context's bit for bit.
int y_metric(Ctx* c, int which, const double* passed, const double** dev) {
  *dev = nullptr;
  if (c->st.istret == 0) return X3D_OK;
  const dvec& v = (which == 0) ? c->st.ppy : c->st.ppyi;
  if (passed && std::memcmp(passed, v.data(), v.size() * sizeof(double)) != 0) return X3D_ERR_COEF;
  const double* d = nullptr;
  int rc = stretch_device(c, &d);
  if (rc != X3D_OK) return rc;
  *dev = d + (size_t)which * c->grid.ny;
  return X3D_OK;
}

// Operators along the grid axis with full (n) extents.
int colloc(x3d_ctx* h, int axis, int kind, double* t, const double* u, const double* f, const double* s,
           const double* w, int nx, int ny, int nz, int npaire, void* st, const double* pp = nullptr) {
  if (!h) return X3D_ERR_ARG;
  Ctx* c = C(h);
  if (nx != c->grid.nx || ny != c->grid.ny || nz != c->grid.nz) return X3D_ERR_SHAPE;
  if (npaire != 0 && npaire != 1) return X3D_ERR_ARG;
  int cs = 0;
  int rc = resolve_set(c, axis, kind, npaire, f, s, w, &cs);
  if (rc != X3D_OK) return rc;
  const int dims[3] = {nx, ny, nz};
  return run_op<double>(h, axis, kind, npaire, cs, t, u, dims, st, pp);
}

int colloc32(x3d_ctx* h, int axis, int kind, float* t, const float* u, int nx, int ny, int nz, int npaire,
             void* st) {
  if (!h) return X3D_ERR_ARG;
  Ctx* c = C(h);
  if (nx != c->grid.nx || ny != c->grid.ny || nz != c->grid.nz) return X3D_ERR_SHAPE;
  const int dims[3] = {nx, ny, nz};
  return run_op<float>(h, axis, kind, npaire, default_coefset(kind, npaire), t, u, dims, st);
}

// Staggered operator: dims_in are the input extents.
int stag(x3d_ctx* h, int axis, int kind, double* t, const double* u, const double* f1, const double* s1,
         const double* w1, const double* f2, const double* s2, const double* w2, const int* dims_in, int npaire,
         void* st, const double* pp = nullptr) {
  if (!h) return X3D_ERR_ARG;
  Ctx* c = C(h);
  if (npaire != 0 && npaire != 1) return X3D_ERR_ARG;
  int cs = default_coefset(kind, npaire);
  const AxisCoef& a = c->ax[axis];
  // p->v operators take two sets: the non-periodic one first, the periodic one second.
  const bool pv = (kind == K_DPV || kind == K_IPV);
  const double *f = f1, *s = s1, *w = w1;
  if (pv && a.periodic) { f = f2; s = s2; w = w2; }
  if (f || s || w) {
    if (pv && a.periodic) {
      int fi, si, wi;
      coef_indices(a, kind, 0, &fi, &si, &wi);
      const size_t n = a.vecs[fi].size() * sizeof(double);
      if (!f || !s || !w || std::memcmp(f, a.vecs[fi].data(), n) || std::memcmp(s, a.vecs[si].data(), n) ||
          std::memcmp(w, a.vecs[wi].data(), n))
        return X3D_ERR_COEF;
    } else {
      int rc = resolve_set(c, axis, kind, npaire, f, s, w, &cs);
      if (rc != X3D_OK) return rc;
    }
  }
  return run_op<double>(h, axis, kind, npaire, cs, t, u, dims_in, st, pp);
}

}  // namespace

extern "C" {

const char* x3d_last_cuda_error(void) {
  return g_last_cuda == cudaSuccess ? "no CUDA error recorded" : cudaGetErrorString(g_last_cuda);
}

const char* x3d_strerror(int s) {
  switch (s) {
    case X3D_OK: return "ok";
    case X3D_ERR_ARG: return "invalid argument";
    case X3D_ERR_SHAPE: return "array extents do not match the grid";
    case X3D_ERR_BC: return "unsupported boundary condition / parity combination";
    case X3D_ERR_DTYPE: return "precision not available";
    case X3D_ERR_CUDA: return "CUDA runtime error";
    case X3D_ERR_COEF: return "coefficient vectors match no set of this context";
    case X3D_ERR_UNSUPPORTED: return "option outside the implemented scope";
    case X3D_ERR_NOMEM: return "device allocation failed";
    case X3D_ERR_STATE: return "solver state error";
    case X3D_ERR_SCRATCH: return "problem larger than the fixed scratch of the allocation-free entry point";
  }
  return "unknown status";
}

int x3d_ctx_create(const x3d_grid* g, const x3d_numopts* o, x3d_ctx** out) {
  if (!g || !o || !out) return X3D_ERR_ARG;
  *out = nullptr;
  if (g->nx < 8 || g->ny < 8 || g->nz < 8) return X3D_ERR_SHAPE;
  if (!(g->xlx > 0) || !(g->yly > 0) || !(g->zlz > 0)) return X3D_ERR_ARG;
  std::unique_ptr<Ctx> c(new Ctx());
  c->grid = *g;
  c->opts = *o;
  // Without a usable device the context still builds its host-side tables
  // (x3d_get_coeffs works); every device call then fails with X3D_ERR_CUDA.
  if (cudaGetDevice(&c->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) {
    cudaGetLastError();
    c->device = -1;
    c->num_sms = 1;
  }
  int rc = build_axis(c->ax[0], g->nx, g->xlx, g->nclx1, g->nclxn, *o);
  if (rc == X3D_OK) rc = build_axis(c->ax[1], g->ny, g->yly, g->ncly1, g->nclyn, *o);
  if (rc == X3D_OK) rc = build_axis(c->ax[2], g->nz, g->zlz, g->nclz1, g->nclzn, *o);
  if (rc == X3D_OK) rc = build_stretch(*g, c->ax[1], c->st);
  if (rc != X3D_OK) return rc;
  *out = reinterpret_cast<x3d_ctx*>(c.release());
  return X3D_OK;
}

int x3d_ctx_destroy(x3d_ctx* h) {
  if (!h) return X3D_ERR_ARG;
  delete C(h);
  return X3D_OK;
}

int x3d_get_coeffs(const x3d_ctx* h, int axis, int which, double* out, int capacity) {
  if (!h || !out || axis < 0 || axis > 2 || which < 0 || which >= X3D_COEF_COUNT) return X3D_ERR_ARG;
  const dvec& v = reinterpret_cast<const Ctx*>(h)->ax[axis].vecs[which];
  if ((int)v.size() > capacity) return X3D_ERR_ARG;
  std::memcpy(out, v.data(), v.size() * sizeof(double));
  return (int)v.size();
}

int x3d_apply(x3d_ctx* h, int axis, int op, int npaire, int coefset, int dtype, void* t, const void* u,
              const int* dims_in, void* stream) {
  if (!h || !dims_in) return X3D_ERR_ARG;
  if (coefset == -1) coefset = default_coefset(op, npaire);
  if (coefset != 0 && coefset != 1) return X3D_ERR_ARG;
  if (dtype == 0) return run_op<double>(h, axis, op, npaire, coefset, (double*)t, (const double*)u, dims_in, stream);
  if (dtype == 1) return run_op<float>(h, axis, op, npaire, coefset, (float*)t, (const float*)u, dims_in, stream);
  return X3D_ERR_DTYPE;
}

int x3d_conv_diff_f32(x3d_ctx* h, int axis, int q, float* out, const float* uj, const float* uq, const float* a1,
                      float nu, const int* dims, void* st) {
  if (!h || !out || !uj || !uq || !dims || axis < 0 || axis > 2 || q < 0 || q > 2) return X3D_ERR_ARG;
  Ctx* c = C(h);
  if (dims[0] != c->grid.nx || dims[1] != c->grid.ny || dims[2] != c->grid.nz) return X3D_ERR_SHAPE;
  if (axis == 1 && c->st.istret != 0) return X3D_ERR_UNSUPPORTED;
  const int pu = (q == axis) ? 0 : 1;  // parity of d_j u_q (momentum_rhs_eq's npaire)
  OpPlan *pA = nullptr, *pB = nullptr, *pC = nullptr;
  int rc = get_plan(c, axis, K_DER1, 1 - pu, default_coefset(K_DER1, 1 - pu), &pA);
  if (rc == X3D_OK) rc = get_plan(c, axis, K_DER1, pu, default_coefset(K_DER1, pu), &pB);
  if (rc == X3D_OK) rc = get_plan(c, axis, K_DER2, pu, default_coefset(K_DER2, pu), &pC);
  if (rc != X3D_OK) return rc;
  return rhs_axis_fast(c, pA, pB, pC, out, uj, uq, a1, nu, dims, (cudaStream_t)st);
}

int x3d_plan_info(x3d_ctx* h, int axis, int op, int npaire, int coefset, double* scalars, double* vecs,
                  double* brows) {
  if (!h) return X3D_ERR_ARG;
  if (coefset == -1) coefset = default_coefset(op, npaire);
  if (coefset != 0 && coefset != 1 || (npaire != 0 && npaire != 1)) return X3D_ERR_ARG;
  return plan_info(C(h), axis, op, npaire, coefset, scalars, vecs, brows);
}

// ---- derivatives and filters -----------------------------------------------
int x3d_derx(x3d_ctx* h, double* tx, const double* ux, double*, double*, const double* ffx, const double* fsx,
             const double* fwx, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 0, K_DER1, tx, ux, ffx, fsx, fwx, nx, ny, nz, npaire, st);
}
int x3d_dery(x3d_ctx* h, double* ty, const double* uy, double*, double*, const double* ffy, const double* fsy,
             const double* fwy, const double* ppy, int nx, int ny, int nz, int npaire, double, void* st) {
  if (!h) return X3D_ERR_ARG;
  const double* pp = nullptr;
  int rc = y_metric(C(h), 0, ppy, &pp);
  if (rc != X3D_OK) return rc;
  return colloc(h, 1, K_DER1, ty, uy, ffy, fsy, fwy, nx, ny, nz, npaire, st, pp);
}
int x3d_derz(x3d_ctx* h, double* tz, const double* uz, double*, double*, const double* ffz, const double* fsz,
             const double* fwz, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 2, K_DER1, tz, uz, ffz, fsz, fwz, nx, ny, nz, npaire, st);
}
int x3d_derxx(x3d_ctx* h, double* tx, const double* ux, double*, double*, const double* sfx, const double* ssx,
              const double* swx, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 0, K_DER2, tx, ux, sfx, ssx, swx, nx, ny, nz, npaire, st);
}
int x3d_deryy(x3d_ctx* h, double* ty, const double* uy, double*, double*, const double* sfy, const double* ssy,
              const double* swy, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 1, K_DER2, ty, uy, sfy, ssy, swy, nx, ny, nz, npaire, st);
}
int x3d_derzz(x3d_ctx* h, double* tz, const double* uz, double*, double*, const double* sfz, const double* ssz,
              const double* swz, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 2, K_DER2, tz, uz, sfz, ssz, swz, nx, ny, nz, npaire, st);
}
int x3d_filx(x3d_ctx* h, double* tx, const double* ux, double*, double*, const double* f, const double* s,
             const double* w, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 0, K_FIL, tx, ux, f, s, w, nx, ny, nz, npaire, st);
}
int x3d_fily(x3d_ctx* h, double* ty, const double* uy, double*, double*, const double* f, const double* s,
             const double* w, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 1, K_FIL, ty, uy, f, s, w, nx, ny, nz, npaire, st);
}
int x3d_filz(x3d_ctx* h, double* tz, const double* uz, double*, double*, const double* f, const double* s,
             const double* w, int nx, int ny, int nz, int npaire, double, void* st) {
  return colloc(h, 2, K_FIL, tz, uz, f, s, w, nx, ny, nz, npaire, st);
}

int x3d_derx_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 0, K_DER1, t, u, nx, ny, nz, np, st);
}
int x3d_dery_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 1, K_DER1, t, u, nx, ny, nz, np, st);
}
int x3d_derz_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 2, K_DER1, t, u, nx, ny, nz, np, st);
}
int x3d_derxx_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 0, K_DER2, t, u, nx, ny, nz, np, st);
}
int x3d_deryy_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 1, K_DER2, t, u, nx, ny, nz, np, st);
}
int x3d_derzz_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 2, K_DER2, t, u, nx, ny, nz, np, st);
}
int x3d_filx_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 0, K_FIL, t, u, nx, ny, nz, np, st);
}
int x3d_fily_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 1, K_FIL, t, u, nx, ny, nz, np, st);
}
int x3d_filz_f32(x3d_ctx* h, float* t, const float* u, int nx, int ny, int nz, int np, void* st) {
  return colloc32(h, 2, K_FIL, t, u, nx, ny, nz, np, st);
}

// ---- staggered operators ----------------------------------------------------
int x3d_derxvp(x3d_ctx* h, double* tx, const double* ux, double*, double*, const double* cfx6, const double* csx6,
               const double* cwx6, int nx, int nxm, int ny, int nz, int npaire, void* st) {
  if (!h || nxm != C(h)->ax[0].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, ny, nz};
  return stag(h, 0, K_DVP, tx, ux, cfx6, csx6, cwx6, nullptr, nullptr, nullptr, d, npaire, st);
}
int x3d_interxvp(x3d_ctx* h, double* tx, const double* ux, double*, double*, const double* cifx6,
                 const double* cisx6, const double* ciwx6, int nx, int nxm, int ny, int nz, int npaire, void* st) {
  if (!h || nxm != C(h)->ax[0].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, ny, nz};
  return stag(h, 0, K_IVP, tx, ux, cifx6, cisx6, ciwx6, nullptr, nullptr, nullptr, d, npaire, st);
}
int x3d_derxpv(x3d_ctx* h, double* tx, const double* ux, double*, double*, const double* cfi6, const double* csi6,
               const double* cwi6, const double* cfx6, const double* csx6, const double* cwx6, int nxm, int nx,
               int ny, int nz, int npaire, void* st) {
  if (!h || nxm != C(h)->ax[0].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nxm, ny, nz};
  return stag(h, 0, K_DPV, tx, ux, cfi6, csi6, cwi6, cfx6, csx6, cwx6, d, npaire, st);
}
int x3d_interxpv(x3d_ctx* h, double* tx, const double* ux, double*, double*, const double* cifi6,
                 const double* cisi6, const double* ciwi6, const double* cifx6, const double* cisx6,
                 const double* ciwx6, int nxm, int nx, int ny, int nz, int npaire, void* st) {
  if (!h || nxm != C(h)->ax[0].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nxm, ny, nz};
  return stag(h, 0, K_IPV, tx, ux, cifi6, cisi6, ciwi6, cifx6, cisx6, ciwx6, d, npaire, st);
}
int x3d_interyvp(x3d_ctx* h, double* ty, const double* uy, double*, double*, const double* cify6,
                 const double* cisy6, const double* ciwy6, int nx, int ny, int nym, int nz, int npaire, void* st) {
  if (!h || nym != C(h)->ax[1].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, ny, nz};
  return stag(h, 1, K_IVP, ty, uy, cify6, cisy6, ciwy6, nullptr, nullptr, nullptr, d, npaire, st);
}
int x3d_deryvp(x3d_ctx* h, double* ty, const double* uy, double*, double*, const double* cfy6, const double* csy6,
               const double* cwy6, const double* ppyi, int nx, int ny, int nym, int nz, int npaire, void* st) {
  if (!h || nym != C(h)->ax[1].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const double* pp = nullptr;
  int rc = y_metric(C(h), 3, ppyi, &pp);
  if (rc != X3D_OK) return rc;
  const int d[3] = {nx, ny, nz};
  return stag(h, 1, K_DVP, ty, uy, cfy6, csy6, cwy6, nullptr, nullptr, nullptr, d, npaire, st, pp);
}
int x3d_interypv(x3d_ctx* h, double* ty, const double* uy, double*, double*, const double* cifi6y,
                 const double* cisi6y, const double* ciwi6y, const double* cify6, const double* cisy6,
                 const double* ciwy6, int nx, int nym, int ny, int nz, int npaire, void* st) {
  if (!h || nym != C(h)->ax[1].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, nym, nz};
  return stag(h, 1, K_IPV, ty, uy, cifi6y, cisi6y, ciwi6y, cify6, cisy6, ciwy6, d, npaire, st);
}
int x3d_derypv(x3d_ctx* h, double* ty, const double* uy, double*, double*, const double* cfi6y,
               const double* csi6y, const double* cwi6y, const double* cfy6, const double* csy6,
               const double* cwy6, const double* ppy, int nx, int nym, int ny, int nz, int npaire, void* st) {
  if (!h || nym != C(h)->ax[1].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const double* pp = nullptr;
  int rc = y_metric(C(h), 0, ppy, &pp);
  if (rc != X3D_OK) return rc;
  const int d[3] = {nx, nym, nz};
  return stag(h, 1, K_DPV, ty, uy, cfi6y, csi6y, cwi6y, cfy6, csy6, cwy6, d, npaire, st, pp);
}
int x3d_derzvp(x3d_ctx* h, double* tz, const double* uz, double*, double*, const double* cfz6, const double* csz6,
               const double* cwz6, int nx, int ny, int nz, int nzm, int npaire, void* st) {
  if (!h || nzm != C(h)->ax[2].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, ny, nz};
  return stag(h, 2, K_DVP, tz, uz, cfz6, csz6, cwz6, nullptr, nullptr, nullptr, d, npaire, st);
}
int x3d_interzvp(x3d_ctx* h, double* tz, const double* uz, double*, double*, const double* cifz6,
                 const double* cisz6, const double* ciwz6, int nx, int ny, int nz, int nzm, int npaire, void* st) {
  if (!h || nzm != C(h)->ax[2].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, ny, nz};
  return stag(h, 2, K_IVP, tz, uz, cifz6, cisz6, ciwz6, nullptr, nullptr, nullptr, d, npaire, st);
}
int x3d_derzpv(x3d_ctx* h, double* tz, const double* uz, double*, double*, const double* cfiz6,
               const double* csiz6, const double* cwiz6, const double* cfz6, const double* csz6,
               const double* cwz6, int nx, int ny, int nzm, int nz, int npaire, void* st) {
  if (!h || nzm != C(h)->ax[2].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, ny, nzm};
  (void)nz;
  return stag(h, 2, K_DPV, tz, uz, cfiz6, csiz6, cwiz6, cfz6, csz6, cwz6, d, npaire, st);
}
int x3d_interzpv(x3d_ctx* h, double* tz, const double* uz, double*, double*, const double* cifiz6,
                 const double* cisiz6, const double* ciwiz6, const double* cifz6, const double* cisz6,
                 const double* ciwz6, int nx, int ny, int nzm, int nz, int npaire, void* st) {
  if (!h || nzm != C(h)->ax[2].nm) return h ? X3D_ERR_SHAPE : X3D_ERR_ARG;
  const int d[3] = {nx, ny, nzm};
  (void)nz;
  return stag(h, 2, K_IPV, tz, uz, cifiz6, cisiz6, ciwiz6, cifz6, cisz6, ciwz6, d, npaire, st);
}

// ---- Poisson, transposes, projection pieces ---------------------------------
int x3d_poisson(x3d_ctx* h, double* rhs, void* st) {
  if (!h || !rhs) return X3D_ERR_ARG;
  Ctx* c = C(h);
  if (c->ax[0].periodic && !c->ax[1].periodic && c->ax[2].periodic) return poisson_010(c, rhs, (cudaStream_t)st);
  if (is_11x(c)) return poisson_11x(c, rhs, (cudaStream_t)st);
  return poisson_periodic(c, rhs, 0, (cudaStream_t)st);
}
int x3d_poisson_noalloc(x3d_ctx* h, double* rhs, void* st) {
  if (!h || !rhs) return X3D_ERR_ARG;
  return poisson_periodic_noalloc(C(h), rhs, (cudaStream_t)st);
}
int x3d_poisson_ex(x3d_ctx* h, double* rhs, int precision, void* st) {
  if (!h || !rhs) return X3D_ERR_ARG;
  Ctx* c = C(h);
  if (c->ax[0].periodic && !c->ax[1].periodic && c->ax[2].periodic)
    return precision == 0 ? poisson_010(c, rhs, (cudaStream_t)st) : X3D_ERR_DTYPE;
  if (is_11x(c)) return precision == 0 ? poisson_11x(c, rhs, (cudaStream_t)st) : X3D_ERR_DTYPE;
  return poisson_periodic(c, rhs, precision, (cudaStream_t)st);
}

int x3d_get_stretching(const x3d_ctx* h, int which, double* out, int capacity) {
  if (!h || !out) return X3D_ERR_ARG;
  const Stretch& st = reinterpret_cast<const Ctx*>(h)->st;
  if (which == 8) {
    if (capacity < 1) return X3D_ERR_ARG;
    out[0] = st.alpha;
    return 1;
  }
  const dvec* tab[] = {&st.yp, &st.ypi, &st.ppy, &st.pp2y, &st.pp4y, &st.ppyi, &st.pp2yi, &st.pp4yi};
  if (which < 0 || which > 7) return X3D_ERR_ARG;
  const dvec& v = *tab[which];
  if ((int)v.size() > capacity) return X3D_ERR_ARG;
  std::memcpy(out, v.data(), v.size() * sizeof(double));
  return (int)v.size();
}

static int tcopy(x3d_ctx* h, const double* src, double* dst, long long n, void* st) {
  if (!h || !src || !dst || n < 0) return X3D_ERR_ARG;
  if (src == dst || n == 0) return X3D_OK;
  return cuda_status(cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, (cudaStream_t)st));
}
int x3d_transpose_x_to_y(x3d_ctx* h, const double* s, double* d, long long n, void* st) { return tcopy(h, s, d, n, st); }
int x3d_transpose_y_to_z(x3d_ctx* h, const double* s, double* d, long long n, void* st) { return tcopy(h, s, d, n, st); }
int x3d_transpose_z_to_y(x3d_ctx* h, const double* s, double* d, long long n, void* st) { return tcopy(h, s, d, n, st); }
int x3d_transpose_y_to_x(x3d_ctx* h, const double* s, double* d, long long n, void* st) { return tcopy(h, s, d, n, st); }

}  // extern "C"
