/*
 * x3d_gpu.h -- C ABI of libx3dgpu.so, the GB300 (sm_103a) implementation of
 * Xcompact3d's per-timestep hot path.
 *
 * Every entry point mirrors one reference routine: the same name (prefixed
 * x3d_), the same argument order and meaning, and the same array layout
 * (Fortran column-major, x fastest).  Differences from the Fortran interface,
 * all deliberate:
 *   - a context handle comes first; it owns the grid, the numerical options,
 *     and the coefficient tables already resident in device memory;
 *   - field arguments (t, u) are DEVICE pointers; the work arrays r and s that
 *     the Fortran interface passes are accepted and ignored (may be NULL): the
 *     Sherman-Morrison vector is data-independent and lives in the context;
 *   - coefficient-vector arguments (ff, fs, fw, ...) are HOST pointers to the
 *     caller's copies (as a Fortran caller has them) or NULL.  When given, they
 *     must match one of the context's coefficient sets bit for bit, otherwise
 *     the call returns X3D_ERR_COEF; NULL selects the set the reference's
 *     callers use for that parity (npaire=1 -> the "p" set);
 *   - the trailing `stream` is a cudaStream_t (NULL = legacy default stream);
 *     every call is stream-ordered and asynchronous;
 *   - every call returns an int status (X3D_OK or a negative X3D_ERR_*)
 *     instead of aborting.
 * Thread safety: one context per host thread; no global mutable state.
 *
 * The _f32 variants are the single-precision build of the same routine
 * (reference built without -DDOUBLE_PREC): float fields, float coefficients.
 */
#ifndef X3D_GPU_H
#define X3D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  X3D_OK = 0,
  X3D_ERR_ARG = -1,         /* NULL handle/pointer or invalid enum value      */
  X3D_ERR_SHAPE = -2,       /* dims do not match the context's grid           */
  X3D_ERR_BC = -3,          /* unsupported boundary-condition / parity combo  */
  X3D_ERR_DTYPE = -4,       /* precision not available for this routine       */
  X3D_ERR_CUDA = -5,        /* a CUDA runtime call failed                     */
  X3D_ERR_COEF = -6,        /* coefficient vectors match no context set       */
  X3D_ERR_UNSUPPORTED = -7, /* option outside the implemented scope           */
  X3D_ERR_NOMEM = -8,       /* device allocation failed                       */
  X3D_ERR_STATE = -9,       /* solver not initialised / numerical blow-up     */
  X3D_ERR_SCRATCH = -10     /* too large for the allocation-free entry point  */
};

typedef struct x3d_ctx x3d_ctx;
typedef struct x3d_solver x3d_solver;
typedef struct x3d_mlp x3d_mlp;

/* Grid: the BasicParam namelist subset (src/parameters.f90:45-90).
 * ncl: 0 periodic, 1 free-slip, 2 Dirichlet. */
typedef struct {
  int nx, ny, nz;
  double xlx, yly, zlz;
  int nclx1, nclxn, ncly1, nclyn, nclz1, nclzn;
  int istret;  /* mesh stretching in y (src/stretching.f90): 0 none, 1 centre,
                  2 both walls, 3 bottom wall; needs a non-periodic y */
  double beta;
} x3d_grid;

/* Numerical options: NumOptions subset (src/parameters.f90; defaults in
 * parameter_defaults). */
typedef struct {
  int ifirstder;       /* 1 or 4 (6th-order compact)                       */
  int isecondder;      /* 1, 4 or 5 (hyperviscous)                         */
  int ipinter;         /* 1, 2 or 3                                        */
  double filter_alpha; /* alpha_f of the compact filter (fpi2 / C_filter)  */
  double nu0nu, cnu;   /* hyperviscous parameters (isecondder=5)           */
} x3d_numopts;

/* --- context --------------------------------------------------------------
 * Replaces init-time setup: schemes() (src/schemes.f90:7-409), filter()
 * (src/filters.f90:5-59) and decomp_2d_poisson_init (src/poisson.f90:73-255).
 * Selects the current CUDA device's tables; all later calls must run on that
 * device. */
int x3d_ctx_create(const x3d_grid* grid, const x3d_numopts* opts, x3d_ctx** out);
int x3d_ctx_destroy(x3d_ctx* ctx);
const char* x3d_strerror(int status);
/* Text of the CUDA runtime error behind the calling thread's most recent
 * X3D_ERR_CUDA status (diagnostics; no counterpart in the reference). */
const char* x3d_last_cuda_error(void);

/* Host copy of a coefficient vector, so a Fortran or C caller can pass the
 * same arrays the reference passes.  axis 0..2; `which` uses the numbering of
 * X3D_COEF_* below; returns the vector length or a negative status. */
enum {
  X3D_COEF_FF = 0, X3D_COEF_FS, X3D_COEF_FW, X3D_COEF_FFP, X3D_COEF_FSP, X3D_COEF_FWP,
  X3D_COEF_SF, X3D_COEF_SS, X3D_COEF_SW, X3D_COEF_SFP, X3D_COEF_SSP, X3D_COEF_SWP,
  X3D_COEF_FIFF, X3D_COEF_FIFS, X3D_COEF_FIFW, X3D_COEF_FIFFP, X3D_COEF_FIFSP, X3D_COEF_FIFWP,
  X3D_COEF_CF6, X3D_COEF_CS6, X3D_COEF_CW6,
  X3D_COEF_CIF6, X3D_COEF_CIS6, X3D_COEF_CIW6,
  X3D_COEF_CIFP6, X3D_COEF_CISP6, X3D_COEF_CIWP6,
  X3D_COEF_CFIP6, X3D_COEF_CSIP6, X3D_COEF_CWIP6,
  X3D_COEF_CIFIP6, X3D_COEF_CISIP6, X3D_COEF_CIWIP6,
  X3D_COEF_CFI6, X3D_COEF_CSI6, X3D_COEF_CWI6,
  X3D_COEF_CIFI6, X3D_COEF_CISI6, X3D_COEF_CIWI6,
  X3D_COEF_CFP6, X3D_COEF_CSP6, X3D_COEF_CWP6,
  X3D_COEF_COUNT
};
int x3d_get_coeffs(const x3d_ctx* ctx, int axis, int which, double* out, int capacity);

/* --- compact first/second derivatives --------------------------------------
 * DERIVATIVE_X / _Y / _YY / _Z interfaces, src/module_param.f90:135-170;
 * implementations src/derive.f90:7-3792 (derx_00 ... derzz_22, bound by BC in
 * src/schemes.f90:30-64).  lind is used by the reference only for IBM and is
 * ignored.  ppy (dery only) is applied when the grid is stretched (istret !=
 * 0, src/derive.f90:409-418): the result is multiplied by the context's ppy;
 * a ppy passed by the caller must equal it bit for bit (else X3D_ERR_COEF),
 * NULL takes the context's.  deryvp takes ppyi and derypv ppy the same way. */
int x3d_derx(x3d_ctx* ctx, double* tx, const double* ux, double* rx, double* sx, const double* ffx,
             const double* fsx, const double* fwx, int nx, int ny, int nz, int npaire, double lind,
             void* stream);
int x3d_dery(x3d_ctx* ctx, double* ty, const double* uy, double* ry, double* sy, const double* ffy,
             const double* fsy, const double* fwy, const double* ppy, int nx, int ny, int nz, int npaire,
             double lind, void* stream);
int x3d_derz(x3d_ctx* ctx, double* tz, const double* uz, double* rz, double* sz, const double* ffz,
             const double* fsz, const double* fwz, int nx, int ny, int nz, int npaire, double lind,
             void* stream);
int x3d_derxx(x3d_ctx* ctx, double* tx, const double* ux, double* rx, double* sx, const double* sfx,
              const double* ssx, const double* swx, int nx, int ny, int nz, int npaire, double lind,
              void* stream);
int x3d_deryy(x3d_ctx* ctx, double* ty, const double* uy, double* ry, double* sy, const double* sfy,
              const double* ssy, const double* swy, int nx, int ny, int nz, int npaire, double lind,
              void* stream);
int x3d_derzz(x3d_ctx* ctx, double* tz, const double* uz, double* rz, double* sz, const double* sfz,
              const double* ssz, const double* swz, int nx, int ny, int nz, int npaire, double lind,
              void* stream);

/* --- compact filters --------------------------------------------------------
 * FILTER_X / _Y / _Z interfaces, src/module_param.f90:202-226; implementations
 * src/filters.f90:221-1377 (filx_00 ... filz_22). */
int x3d_filx(x3d_ctx* ctx, double* tx, const double* ux, double* rx, double* fisx, const double* fiffx,
             const double* fifsx, const double* fifwx, int nx, int ny, int nz, int npaire, double lind,
             void* stream);
int x3d_fily(x3d_ctx* ctx, double* ty, const double* uy, double* ry, double* fisy, const double* fiffy,
             const double* fifsy, const double* fifwy, int nx, int ny, int nz, int npaire, double lind,
             void* stream);
int x3d_filz(x3d_ctx* ctx, double* tz, const double* uz, double* rz, double* fisz, const double* fiffz,
             const double* fifsz, const double* fifwz, int nx, int ny, int nz, int npaire, double lind,
             void* stream);

/* --- staggered (velocity <-> pressure mesh) operators -------------------------
 * src/derive.f90:3796-5615.  Argument lists follow the Fortran subroutines. */
int x3d_derxvp(x3d_ctx* ctx, double* tx, const double* ux, double* rx, double* sx, const double* cfx6,
               const double* csx6, const double* cwx6, int nx, int nxm, int ny, int nz, int npaire,
               void* stream);
int x3d_interxvp(x3d_ctx* ctx, double* tx, const double* ux, double* rx, double* sx, const double* cifx6,
                 const double* cisx6, const double* ciwx6, int nx, int nxm, int ny, int nz, int npaire,
                 void* stream);
int x3d_derxpv(x3d_ctx* ctx, double* tx, const double* ux, double* rx, double* sx, const double* cfi6,
               const double* csi6, const double* cwi6, const double* cfx6, const double* csx6,
               const double* cwx6, int nxm, int nx, int ny, int nz, int npaire, void* stream);
int x3d_interxpv(x3d_ctx* ctx, double* tx, const double* ux, double* rx, double* sx, const double* cifi6,
                 const double* cisi6, const double* ciwi6, const double* cifx6, const double* cisx6,
                 const double* ciwx6, int nxm, int nx, int ny, int nz, int npaire, void* stream);
int x3d_interyvp(x3d_ctx* ctx, double* ty, const double* uy, double* ry, double* sy, const double* cify6,
                 const double* cisy6, const double* ciwy6, int nx, int ny, int nym, int nz, int npaire,
                 void* stream);
int x3d_deryvp(x3d_ctx* ctx, double* ty, const double* uy, double* ry, double* sy, const double* cfy6,
               const double* csy6, const double* cwy6, const double* ppyi, int nx, int ny, int nym, int nz,
               int npaire, void* stream);
int x3d_interypv(x3d_ctx* ctx, double* ty, const double* uy, double* ry, double* sy, const double* cifi6y,
                 const double* cisi6y, const double* ciwi6y, const double* cify6, const double* cisy6,
                 const double* ciwy6, int nx, int nym, int ny, int nz, int npaire, void* stream);
int x3d_derypv(x3d_ctx* ctx, double* ty, const double* uy, double* ry, double* sy, const double* cfi6y,
               const double* csi6y, const double* cwi6y, const double* cfy6, const double* csy6,
               const double* cwy6, const double* ppy, int nx, int nym, int ny, int nz, int npaire,
               void* stream);
int x3d_derzvp(x3d_ctx* ctx, double* tz, const double* uz, double* rz, double* sz, const double* cfz6,
               const double* csz6, const double* cwz6, int nx, int ny, int nz, int nzm, int npaire,
               void* stream);
int x3d_interzvp(x3d_ctx* ctx, double* tz, const double* uz, double* rz, double* sz, const double* cifz6,
                 const double* cisz6, const double* ciwz6, int nx, int ny, int nz, int nzm, int npaire,
                 void* stream);
int x3d_derzpv(x3d_ctx* ctx, double* tz, const double* uz, double* rz, double* sz, const double* cfiz6,
               const double* csiz6, const double* cwiz6, const double* cfz6, const double* csz6,
               const double* cwz6, int nx, int ny, int nzm, int nz, int npaire, void* stream);
int x3d_interzpv(x3d_ctx* ctx, double* tz, const double* uz, double* rz, double* sz, const double* cifiz6,
                 const double* cisiz6, const double* ciwiz6, const double* cifz6, const double* cisz6,
                 const double* ciwz6, int nx, int ny, int nzm, int nz, int npaire, void* stream);

/* --- generic operator entry (used by the per-routine wrappers above) --------
 * op: 0 der1, 1 der2, 2 filter, 3 d(v->p), 4 interp(v->p), 5 d(p->v),
 * 6 interp(p->v).  axis 0..2.  dims_in = extents of u (nx_in, ny_in, nz_in).
 * dtype: 0 = float64, 1 = float32.  coefset: -1 = default for npaire,
 * 0 = plain set, 1 = "p" set. */
int x3d_apply(x3d_ctx* ctx, int axis, int op, int npaire, int coefset, int dtype, void* t, const void* u,
              const int* dims_in, void* stream);

/* One direction's share of the momentum right-hand side of component u_q,
 * binary32, periodic lines (src/transeq.f90:73-591: the convective term in
 * skew-symmetric form plus the viscous term along axis j = axis):
 *   out = nu d_jj u_q + a1 - (d_j(u_j u_q) + u_j d_j u_q) / 2
 * npaire is (q == axis ? 0 : 1) for d_j u_q and d_jj u_q and the reverse for
 * the product, as momentum_rhs_eq calls them.  The three solves of a line run
 * in one kernel, reading u_j, u_q and a1 once and writing out once.  a1 may be
 * null (zero) or alias out.  dims = (nx, ny, nz) of the context.  Returns
 * X3D_ERR_UNSUPPORTED where the fused kernel does not apply: a non-periodic
 * axis, a stretched y axis, or a line length other than 16 * {8, 16, 32}
 * (32 * {4, 8, 16} also for x).  No reference counterpart as one call: it
 * replaces the derx/dery/derz + derxx/deryy/derzz sequence of one direction in
 * momentum_rhs_eq. */
int x3d_conv_diff_f32(x3d_ctx* ctx, int axis, int q, float* out, const float* uj, const float* uq,
                      const float* a1, float nu, const int* dims, void* stream);

/* Host-side description of the plan x3d_apply uses for (axis, op, npaire,
 * coefset): the line kernel's interior coefficients, Thomas factors,
 * chunked-solve fix-up factors, Sherman-Morrison vector and boundary-row
 * table (layout documented in incompact3d_gb300/csrc/x3d_internal.h);
 * scalars[13] is 1 when the periodic system is the circulant [alpha, 1,
 * alpha] and the circulant-form kernels solve it.  No device work; returns
 * the output line length or a negative status.  Has no counterpart in the
 * reference (diagnostics). */
int x3d_plan_info(x3d_ctx* ctx, int axis, int op, int npaire, int coefset, double* scalars, double* vecs,
                  double* brows);

/* --- single-precision builds of the derivative / filter routines ---------- */
int x3d_derx_f32(x3d_ctx* ctx, float* tx, const float* ux, int nx, int ny, int nz, int npaire, void* stream);
int x3d_dery_f32(x3d_ctx* ctx, float* ty, const float* uy, int nx, int ny, int nz, int npaire, void* stream);
int x3d_derz_f32(x3d_ctx* ctx, float* tz, const float* uz, int nx, int ny, int nz, int npaire, void* stream);
int x3d_derxx_f32(x3d_ctx* ctx, float* tx, const float* ux, int nx, int ny, int nz, int npaire, void* stream);
int x3d_deryy_f32(x3d_ctx* ctx, float* ty, const float* uy, int nx, int ny, int nz, int npaire, void* stream);
int x3d_derzz_f32(x3d_ctx* ctx, float* tz, const float* uz, int nx, int ny, int nz, int npaire, void* stream);
int x3d_filx_f32(x3d_ctx* ctx, float* tx, const float* ux, int nx, int ny, int nz, int npaire, void* stream);
int x3d_fily_f32(x3d_ctx* ctx, float* ty, const float* uy, int nx, int ny, int nz, int npaire, void* stream);
int x3d_filz_f32(x3d_ctx* ctx, float* tz, const float* uz, int nx, int ny, int nz, int npaire, void* stream);

/* --- Poisson solve ------------------------------------------------------------
 * poisson(rhs) procedure pointer, src/poisson.f90:57-62, chosen from the
 * boundary conditions as decomp_2d_poisson_init does (src/poisson.f90:97-107):
 *   all periodic                 -> poisson_000, src/poisson.f90:298-410;
 *   x, z periodic, y walls       -> poisson_010, src/poisson.f90:665-1013
 *     (cosine transform in y; on a stretched mesh, istret 1 or 2, the two
 *     pentadiagonal systems of matrice_refinement, src/poisson.f90:1814-2113,
 *     solved as inversion5_v1, src/tools.f90:1225-1362);
 *   x, y free-slip (ncl 1/1), z free-slip or periodic
 *                                -> poisson_11x, src/poisson.f90:1019-1465
 *     (uniform mesh; the even/odd reorders and half-cell cosine combinations
 *     along x and y, and along z when it is free-slip).
 * rhs (nxm,nym,nzm) in device memory is overwritten by the solution.
 * precision (poisson_000 only): 0 = FP64 FFT, 1 = FP32 FFT, 2 = double-float
 * FFT (each real carried as a hi+lo pair of binary32, ~48-bit significand,
 * computed on the FP32 pipes).  poisson_010 and poisson_11x run in FP64. */
int x3d_poisson(x3d_ctx* ctx, double* rhs, void* stream);
int x3d_poisson_ex(x3d_ctx* ctx, double* rhs, int precision, void* stream);

/* Allocation-free form of x3d_poisson (FP64 FFT), for callers that cannot
 * allocate device memory when they solve: codes whose device memory is
 * reserved up front in their own pool and that treat any later allocation as
 * an error.  x3d_poisson allocates its spectrum and tables in the context on
 * first use; this entry point instead uses one fixed array of
 * X3D_NOALLOC_SCRATCH_BYTES in the library's device image (held by every GPU
 * that loads the library until the process exits) and calls no allocating
 * routine.  The spectrum needs (nx/2+1)*ny*nz*16 bytes plus small tables;
 * larger grids return X3D_ERR_SCRATCH (e.g. 128^3 fits, 256^3 does not).  The
 * array is shared by every call from any context or stream and keeps the last
 * call's contents (each call rewrites everything it reads), so calls that
 * overlap on the GPU race.  The first call on each device looks up the
 * array's device address with that device current; make that first call
 * before any stream capture.  Same argument meaning and result as
 * x3d_poisson.  No counterpart in the reference. */
#define X3D_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int x3d_poisson_noalloc(x3d_ctx* ctx, double* rhs, void* stream);

/* Host copy of the y-mesh metrics computed at context creation (module
 * variables yp, ypi, ppy, pp2y, pp4y, ppyi, pp2yi, pp4yi of
 * src/variables.f90:1294-1336 / src/stretching.f90:92-270): which = 0..7 in
 * that order (ny values each), 8 = the mapping constant alpha.  Returns the
 * number of values written. */
int x3d_get_stretching(const x3d_ctx* ctx, int which, double* out, int capacity);

/* --- 2DECOMP transposes ------------------------------------------------------
 * transpose_x_to_y / y_to_z / z_to_y / y_to_x of 2DECOMP&FFT.  On one GPU the
 * X-, Y- and Z-pencils are the same (nx,ny,nz) array, so each is a device copy
 * (or nothing when src == dst).  n = number of elements. */
int x3d_transpose_x_to_y(x3d_ctx* ctx, const double* src, double* dst, long long n, void* stream);
int x3d_transpose_y_to_z(x3d_ctx* ctx, const double* src, double* dst, long long n, void* stream);
int x3d_transpose_z_to_y(x3d_ctx* ctx, const double* src, double* dst, long long n, void* stream);
int x3d_transpose_y_to_x(x3d_ctx* ctx, const double* src, double* dst, long long n, void* stream);

/* --- projection pieces ---------------------------------------------------------
 * divergence (nlock=1, src/navier.f90:257-372), gradp (src/navier.f90:386-499),
 * cor_vel (src/navier.f90:206-249).  Device pointers; pp3 is (nxm,nym,nzm). */
int x3d_divergence(x3d_ctx* ctx, double* pp3, const double* ux, const double* uy, const double* uz,
                   void* stream);
int x3d_gradp(x3d_ctx* ctx, double* px, double* py, double* pz, const double* pp3, void* stream);
/* binary32 builds of divergence (FP64 result, as the mixed-precision step
 * hands it to the Poisson solve) and gradp, same staggered-operator sequence;
 * on periodic lines of 128, 256 or 512 points they run the circulant-form
 * kernels with the y / z sums and pairs fused.  Uniform meshes only
 * (X3D_ERR_UNSUPPORTED for istret != 0). */
int x3d_divergence_f32(x3d_ctx* ctx, double* pp3, const float* ux, const float* uy, const float* uz, void* stream);
int x3d_gradp_f32(x3d_ctx* ctx, float* px, float* py, float* pz, const float* pp3, void* stream);
int x3d_cor_vel(x3d_ctx* ctx, double* ux, double* uy, double* uz, const double* px, const double* py,
                const double* pz, void* stream);

/* --- incompressible solver (the time loop body of src/xcompact3d.f90:29-102):
 * calculate_transeq_rhs (src/transeq.f90:20-591), int_time
 * (src/time_integrators.f90), pre_correc, solve_poisson + cor_vel
 * (src/navier.f90).  The solver owns u, v, w, the time-integrator history and
 * the work fields, all resident in device memory.
 * Geometries: triply periodic (poisson_000), or the channel: x and z
 * periodic with no-slip walls at both y ends (ncly1 = nclyn = 2, optionally a
 * stretched y mesh, poisson_010), FP64 only.
 * precision: X3D_PREC_FP64 computes everything in binary64;
 * X3D_PREC_MIXED runs derivatives, convective/viscous terms and the staggered
 * operators in binary32, keeps the velocity, the time-integrator history and
 * accumulation, and the Poisson solve in binary64. */
enum { X3D_PREC_FP64 = 0, X3D_PREC_MIXED = 1 };
typedef struct {
  int itimescheme; /* 3 = AB3 (Euler, AB2 start-up), 5 = RK3 */
  double dt;
  double xnu;      /* 1/Re */
  int precision;   /* X3D_PREC_* */
} x3d_solver_opts;

int x3d_solver_create(x3d_ctx* ctx, const x3d_solver_opts* opts, x3d_solver** out);
int x3d_solver_destroy(x3d_solver* s);
/* Copy the velocity in or out.  on_device: 1 = device pointers, 0 = host. */
int x3d_solver_set_velocity(x3d_solver* s, const double* ux, const double* uy, const double* uz, int on_device);
int x3d_solver_get_velocity(x3d_solver* s, double* ux, double* uy, double* uz, int on_device);
/* Asynchronous forms for page-locked host buffers (cudaHostAlloc /
 * pin_memory; X3D_ERR_ARG otherwise), stream-ordered with x3d_solver_step on
 * the same stream: set_velocity_async replaces the velocity after the work
 * already queued on `stream` and before any later step, keeping the time
 * level and the integrator history (a round trip of the state through host
 * memory, unlike x3d_solver_set_velocity, which restarts the time
 * integration); get_velocity_async writes the velocity as of the work queued
 * on `stream`.  Read-outs run in the order u, v, w on one transfer stream,
 * write-ins on another, each after its own component's read-out, so in a
 * set / step / get loop on shared buffers the write-in of one component
 * overlaps the read-out of the next.  The host buffers are complete after x3d_solver_sync (or
 * a device synchronisation).  No reference counterpart (the reference keeps
 * its fields in host memory). */
int x3d_solver_set_velocity_async(x3d_solver* s, const double* ux, const double* uy, const double* uz,
                                  void* stream);
int x3d_solver_get_velocity_async(x3d_solver* s, double* ux, double* uy, double* uz, void* stream);
int x3d_solver_sync(x3d_solver* s);
/* Initial condition of init_tgv (src/Case-TGV.f90:25-107), iin=1. */
int x3d_solver_init_tgv(x3d_solver* s);
/* Advance nsteps time steps (each with its sub-steps), stream-ordered. */
int x3d_solver_step(x3d_solver* s, int nsteps, void* stream);
/* TGV statistics of postprocess_tgv (src/Case-TGV.f90:189-477):
 * out = {E_k, eps (strain), eps2 (laplacian), enstrophy}.  Synchronises. */
int x3d_solver_tgv_stats(x3d_solver* s, double* out, void* stream);
/* max |div u| on the pressure mesh (test_flow / divergence nlock=2).  Synchronises. */
int x3d_solver_divmax(x3d_solver* s, double* out, void* stream);
/* Number of kernels this solver launches per time step. */
int x3d_solver_launches_per_step(x3d_solver* s);
/* Channel case (itype = channel, src/Case-Channel.f90): before every sub-step
 * channel_cfr (src/Case-Channel.f90:221-264) shifts u so that the bulk
 * velocity is target_ub (the reference uses 2/3); while the step index is
 * below spinup_time the rotation forcing of momentum_forcing_channel
 * (src/Case-Channel.f90:392-421) with speed wrotation is added.  The no-slip
 * wall values of pre_correc and the wall pressure gradients of gradp are
 * always applied in the channel geometry.  X3D_ERR_BC on a periodic solver. */
int x3d_solver_set_channel(x3d_solver* s, double target_ub, double wrotation, int spinup_time);
/* Explicit LES in the right-hand side (compute_SGS, src/les_models.f90:96-165,
 * iconserv = 0): jles = 1 Smagorinsky (smag, :168-331) with constant smagcst,
 * jles = 3 dynamic Smagorinsky (dynsmag, :333-903; filters with alpha = 0 as
 * its filter(zero) call sets, constant clipped to [0, maxdsmagcst]), 0 off.
 * The force of sgs_mom_nonconservative (:1091-1250) is added to the momentum
 * right-hand side.  FP64 solver only (X3D_ERR_DTYPE otherwise). */
int x3d_solver_set_les(x3d_solver* s, int jles, double smagcst, double maxdsmagcst);
/* Eddy viscosity and SGS force of the current velocity into device arrays of
 * N = nx*ny*nz doubles (for checks and output), stream-ordered. */
int x3d_solver_les_fields(x3d_solver* s, double* nut, double* sgsx, double* sgsy, double* sgsz, void* stream);
/* Restart state (restart, src/tools.f90:205-514): which = 0..2 velocity
 * (ux, uy, uz), 3..5 the previous right-hand side (dux1(:,:,:,2), ... of
 * AB2/AB3), 6..8 the one before (dux1(:,:,:,3), AB3 only), 9 the pressure
 * pp3 on the pressure mesh (nxm*nym*nzm values).  on_device: 1 = device
 * pointer, 0 = host.  X3D_ERR_STATE for a slot the time scheme does not keep. */
int x3d_solver_get_field(x3d_solver* s, int which, double* out, int on_device);
int x3d_solver_set_field(x3d_solver* s, int which, const double* in, int on_device);
/* Completed time steps (itime - 1 of the reference's loop); set it when
 * restarting so that AB3 does not repeat its Euler/AB2 start-up. */
int x3d_solver_get_itime(x3d_solver* s);
int x3d_solver_set_itime(x3d_solver* s, int itime);
/* --- learned SGS closure (no counterpart in the reference; its dynamic
 * Smagorinsky model, jles = 3, is the fallback and the cost baseline) ----------
 * A pointwise MLP (9 velocity-gradient components du_i/dx_j, i-major, + the
 * filter width) -> 64 -> 64 -> 6 tau_ij (xx, yy, zz, xy, xz, yz), GELU, FP32
 * parameters.  Parameters: W1[64][10], b1[64], W2[64][64], b2[64], W3[6][64],
 * b3[6] (x3d_mlp_param_count() floats); scales: 10 input multipliers then 6
 * output multipliers (tau = out_scale * MLP(features * in_scale)).  Only the
 * 10-64-64-6 shape is built. */
int x3d_mlp_create(int nin, int nhidden, int nout, x3d_mlp** out);
int x3d_mlp_destroy(x3d_mlp* m);
int x3d_mlp_param_count(void);
/* Host arrays (either may be NULL); setting resets the Adam state. */
int x3d_mlp_set_params(x3d_mlp* m, const float* params, const float* scales);
int x3d_mlp_get_params(x3d_mlp* m, float* params, float* scales);
/* Y[n][6] = tau for features X[n][10] (device arrays). */
int x3d_mlp_infer(x3d_mlp* m, const float* X, float* Y, long long n, void* stream);
/* One Adam step (lr) on the batch X[n][10] -> T[n][6] (device arrays) with the
 * loss mean_n sum_ij (tau/out_scale - target/out_scale)^2; loss (host, may be
 * NULL, synchronises) receives the loss before the step. */
int x3d_mlp_train_step(x3d_mlp* m, const float* X, const float* T, long long n, float lr, float* loss,
                       void* stream);
/* Inference on the tensor cores (on = 1; default 0 = FP32 CUDA cores): the
 * three layers as tcgen05 MMAs of 128 points, BF16 hi / lo split operands
 * (hi*hi + hi*lo + lo*hi) accumulated in FP32 in tensor memory, within about
 * 1e-4 relative of the FP32 kernel.  Applies to x3d_mlp_infer and to the
 * solver's closure (x3d_solver_set_les_mlp). */
int x3d_mlp_set_tensor_cores(x3d_mlp* m, int on);
/* X3D_ERR_CUDA if a bounded wait inside a tensor-core inference ran out (the
 * kernel then stops and leaves its outputs incomplete), else X3D_OK.
 * Synchronises. */
int x3d_mlp_status(x3d_mlp* m);
/* Add lam * ((Pi_model - Pi_target) / pscale)^2 to the training loss, with the
 * subgrid energy flux Pi = tau_ij S_ij (S from the raw gradient features);
 * lam = 0 (default) is the plain stress loss. */
int x3d_mlp_set_flux_loss(x3d_mlp* m, float lam, float pscale);
/* Box filter of ratio 4 (centred trapezoid 1/2,1,1,1,1/2 over 5 points per
 * direction, periodic) of a fine velocity field (nx,ny,nz) onto the
 * (nx/4,ny/4,nz/4) grid: filtered velocity and tau_ij = (u_i u_j)^f -
 * u_i^f u_j^f (6 consecutive coarse fields in tau).  Device arrays. */
int x3d_box_filter4(const double* ux, const double* uy, const double* uz, int nx, int ny, int nz, double* ubar,
                    double* vbar, double* wbar, double* tau, void* stream);
/* Use the MLP as the solver's SGS model: the force -d_j tau_ij of its
 * stresses joins the right-hand side (FP64 solver; the model is not owned). */
int x3d_solver_set_les_mlp(x3d_solver* s, x3d_mlp* m);
/* Bulk velocity measured by channel_cfr (before its correction) at each
 * sub-step of the last step; returns the number of values.  Synchronises. */
int x3d_solver_bulk_velocity(x3d_solver* s, double* out, int capacity);

#ifdef __cplusplus
}
#endif
#endif /* X3D_GPU_H */
