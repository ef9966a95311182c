// Learned subgrid-stress closure for LES: a pointwise MLP
//   (9 velocity-gradient components + filter width) -> 64 -> 64 -> 6 tau_ij
// with GELU activations and FP32 weights, plus everything needed to train it
// on box-filtered DNS that the solver itself produces:
//   * k_box4_stress: box filter of ratio 4 of a fine velocity field onto the
//     coarse grid (filtered velocity and tau_ij = (u_i u_j)^f - u_i^f u_j^f);
//   * fused inference on feature arrays and directly on the LES gradient
//     fields (one thread per point, weights in shared memory);
//   * training: per-sample forward and backward pass in one kernel, block
//     partial gradients reduced in fixed order, Adam update.
// The dynamic Smagorinsky model of the reference (src/les_models.f90) is the
// fallback and the cost baseline; this closure has no reference counterpart.
#include <cmath>
#include <cstring>
#include <vector>

#include "x3d_internal.h"

namespace x3d {
namespace {

using mlpdim::NI;
using mlpdim::NH;
using mlpdim::NO;
using mlpdim::OW1;
using mlpdim::OB1;
using mlpdim::OW2;
using mlpdim::OB2;
using mlpdim::OW3;
using mlpdim::OB3;
using mlpdim::NPAR;

#define GSTRIDE(i, n) \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// Forward pass of one sample with parameters in shared memory.
__device__ __forceinline__ void mlp_point(const float* P, const float* x, float* y) {
  float h1[NH];
#pragma unroll
  for (int k = 0; k < NH; ++k) {
    float a = P[OB1 + k];
#pragma unroll
    for (int i = 0; i < NI; ++i) a = a + P[OW1 + k * NI + i] * x[i];
    h1[k] = gelu(a);
  }
#pragma unroll
  for (int m = 0; m < NO; ++m) y[m] = P[OB3 + m];
  for (int j = 0; j < NH; ++j) {
    float a = P[OB2 + j];
#pragma unroll
    for (int k = 0; k < NH; ++k) a = a + P[OW2 + j * NH + k] * h1[k];
    const float g = gelu(a);
#pragma unroll
    for (int m = 0; m < NO; ++m) y[m] = y[m] + P[OW3 + m * NH + j] * g;
  }
}

__device__ __forceinline__ void load_params(float* sp, const float* P, const float* sc, int nsc) {
  for (int i = threadIdx.x; i < NPAR; i += blockDim.x) sp[i] = P[i];
  for (int i = threadIdx.x; i < nsc; i += blockDim.x) sp[NPAR + i] = sc[i];
  __syncthreads();
}

// Inference on row-major feature arrays: Y[s] = outscale * MLP(X[s] * inscale).
__global__ void __launch_bounds__(256) k_mlp_infer(const float* P, const float* sc, const float* X, float* Y,
                                                   long long n) {
  extern __shared__ float sp[];
  load_params(sp, P, sc, NI + NO);
  const float* insc = sp + NPAR;
  const float* outsc = insc + NI;
  GSTRIDE(s, n) {
    float x[NI], y[NO];
#pragma unroll
    for (int i = 0; i < NI; ++i) x[i] = X[s * NI + i] * insc[i];
    mlp_point(sp, x, y);
#pragma unroll
    for (int m = 0; m < NO; ++m) Y[s * NO + m] = y[m] * outsc[m];
  }
}

struct G9 {
  const double* g[9];
};
struct T6 {
  double* t[6];
};

// Inference on the LES fields: features are the 9 gradient fields (binary64)
// and the filter width; tau_ij written in binary64.
__global__ void __launch_bounds__(256) k_mlp_les(const float* P, const float* sc, G9 g, float delta, T6 tau,
                                                 long long n) {
  extern __shared__ float sp[];
  load_params(sp, P, sc, NI + NO);
  const float* insc = sp + NPAR;
  const float* outsc = insc + NI;
  GSTRIDE(m, n) {
    float x[NI], y[NO];
#pragma unroll
    for (int i = 0; i < 9; ++i) x[i] = (float)g.g[i][m] * insc[i];
    x[9] = delta * insc[9];
    mlp_point(sp, x, y);
#pragma unroll
    for (int q = 0; q < NO; ++q) tau.t[q][m] = (double)(y[q] * outsc[q]);
  }
}

// Training: 64 samples per block.  Per-sample activations and deltas go to
// padded shared arrays [unit][65]; the block then forms its partial gradient
// (sum over its samples in fixed order) and its partial squared error.
constexpr int TB = 64;
constexpr int PD = TB + 1;

// Optional energy-flux term of the loss: lam * ((Pi_model - Pi_data) / pscale)^2
// with Pi = tau_ij S_ij (S from the raw gradient features), which ties the
// model to the subgrid dissipation the LES needs.
__global__ void __launch_bounds__(TB) k_mlp_grad(const float* P, const float* sc, const float* X, const float* T,
                                                 long long n, float lam, float pscale, float* part, float* lpart) {
  extern __shared__ float sm[];
  float* sp = sm;                  // parameters + scales
  float* xs = sp + NPAR + NI + NO;  // [NI][PD]
  float* h1s = xs + NI * PD;       // [NH][PD]
  float* d1s = h1s + NH * PD;
  float* h2s = d1s + NH * PD;
  float* d2s = h2s + NH * PD;
  float* dys = d2s + NH * PD;      // [NO][PD]
  float* ls = dys + NO * PD;       // [TB]
  for (int i = threadIdx.x; i < NPAR; i += TB) sp[i] = P[i];
  for (int i = threadIdx.x; i < NI + NO; i += TB) sp[NPAR + i] = sc[i];
  __syncthreads();
  const float* insc = sp + NPAR;
  const float* outsc = insc + NI;
  const int t = threadIdx.x;
  const long long s = (long long)blockIdx.x * TB + t;
  const bool ok = s < n;
  float x[NI], a1[NH], h1[NH];
#pragma unroll
  for (int i = 0; i < NI; ++i) x[i] = ok ? X[s * NI + i] * insc[i] : 0.f;
#pragma unroll
  for (int k = 0; k < NH; ++k) {
    float a = sp[OB1 + k];
#pragma unroll
    for (int i = 0; i < NI; ++i) a = a + sp[OW1 + k * NI + i] * x[i];
    a1[k] = a;
    h1[k] = gelu(a);
  }
  float y[NO];
#pragma unroll
  for (int m = 0; m < NO; ++m) y[m] = sp[OB3 + m];
  for (int j = 0; j < NH; ++j) {
    float a = sp[OB2 + j];
#pragma unroll
    for (int k = 0; k < NH; ++k) a = a + sp[OW2 + j * NH + k] * h1[k];
    const float g = gelu(a);
    h2s[j * PD + t] = g;
    d2s[j * PD + t] = gelu_d(a);  // derivative, turned into the delta below
#pragma unroll
    for (int m = 0; m < NO; ++m) y[m] = y[m] + sp[OW3 + m * NH + j] * g;
  }
  // loss: mean over the batch of sum_m (y_m - t_m / outscale_m)^2 [+ flux term]
  float dy[NO], l = 0.f;
#pragma unroll
  for (int m = 0; m < NO; ++m) {
    const float e = ok ? y[m] - T[s * NO + m] / outsc[m] : 0.f;
    l = l + e * e;
    dy[m] = 2.f * e / (float)n;
  }
  if (lam != 0.f && ok) {
    const float* g = X + s * NI;  // raw du_i/dx_j, i-major
    const float S[NO] = {g[0], g[4], g[8], 0.5f * (g[1] + g[3]), 0.5f * (g[2] + g[6]), 0.5f * (g[5] + g[7])};
    float pm = 0.f, pd = 0.f;
#pragma unroll
    for (int m = 0; m < NO; ++m) {
      const float wm = (m < 3) ? 1.f : 2.f;
      pm = pm + wm * (y[m] * outsc[m]) * S[m];
      pd = pd + wm * T[s * NO + m] * S[m];
    }
    const float e = (pm - pd) / pscale;
    l = l + lam * e * e;
#pragma unroll
    for (int m = 0; m < NO; ++m) {
      const float wm = (m < 3) ? 1.f : 2.f;
      dy[m] = dy[m] + 2.f * lam * e * wm * S[m] * outsc[m] / pscale / (float)n;
    }
  }
#pragma unroll
  for (int m = 0; m < NO; ++m) dys[m * PD + t] = dy[m];
  ls[t] = l;
  for (int j = 0; j < NH; ++j) {
    float d = 0.f;
#pragma unroll
    for (int m = 0; m < NO; ++m) d = d + sp[OW3 + m * NH + j] * dy[m];
    d2s[j * PD + t] = d * d2s[j * PD + t];
  }
#pragma unroll
  for (int k = 0; k < NH; ++k) {
    float d = 0.f;
    for (int j = 0; j < NH; ++j) d = d + sp[OW2 + j * NH + k] * d2s[j * PD + t];
    d1s[k * PD + t] = d * gelu_d(a1[k]);
    h1s[k * PD + t] = h1[k];
  }
#pragma unroll
  for (int i = 0; i < NI; ++i) xs[i * PD + t] = x[i];
  __syncthreads();
  // block partial gradients, samples summed in order
  float* out = part + (size_t)blockIdx.x * NPAR;
  for (int p = t; p < NPAR; p += TB) {
    float acc = 0.f;
    if (p < OB1) {
      const int k = p / NI, i = p % NI;
      for (int u = 0; u < TB; ++u) acc = acc + d1s[k * PD + u] * xs[i * PD + u];
    } else if (p < OW2) {
      const int k = p - OB1;
      for (int u = 0; u < TB; ++u) acc = acc + d1s[k * PD + u];
    } else if (p < OB2) {
      const int j = (p - OW2) / NH, k = (p - OW2) % NH;
      for (int u = 0; u < TB; ++u) acc = acc + d2s[j * PD + u] * h1s[k * PD + u];
    } else if (p < OW3) {
      const int j = p - OB2;
      for (int u = 0; u < TB; ++u) acc = acc + d2s[j * PD + u];
    } else if (p < OB3) {
      const int m = (p - OW3) / NH, j = (p - OW3) % NH;
      for (int u = 0; u < TB; ++u) acc = acc + dys[m * PD + u] * h2s[j * PD + u];
    } else {
      const int m = p - OB3;
      for (int u = 0; u < TB; ++u) acc = acc + dys[m * PD + u];
    }
    out[p] = acc;
  }
  if (t == 0) {
    float a = 0.f;
    for (int u = 0; u < TB; ++u) a = a + ls[u];
    lpart[blockIdx.x] = a;
  }
}

// Sum of block partials in block order, then Adam (Kingma & Ba 2015).
__global__ void k_mlp_adam(float* P, float* m1, float* m2, const float* part, int nb, float lr, float b1c, float b2c) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPAR) return;
  float g = 0.f;
  for (int b = 0; b < nb; ++b) g = g + part[(size_t)b * NPAR + p];
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  m1[p] = beta1 * m1[p] + (1.f - beta1) * g;
  m2[p] = beta2 * m2[p] + (1.f - beta2) * g * g;
  const float mh = m1[p] / b1c, vh = m2[p] / b2c;
  P[p] = P[p] - lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_sum(const float* a, int n, float* out) {
  float s = 0.f;
  for (int i = 0; i < n; ++i) s = s + a[i];
  *out = s;
}

// Box filter of ratio 4 onto the coarse grid (centred trapezoidal weights
// 1/2, 1, 1, 1, 1/2 over offsets -2..2, divided by 4, per direction), periodic.
// out: ubar, vbar, wbar, then tau_xx, tau_yy, tau_zz, tau_xy, tau_xz, tau_yz.
__global__ void k_box4_stress(const double* ux, const double* uy, const double* uz, int nx, int ny, int nz, T6 o3,
                              T6 o6) {
  const int mx = nx / 4, my = ny / 4, mz = nz / 4;
  const long long mc = (long long)mx * my * mz;
  const double wt[5] = {0.125, 0.25, 0.25, 0.25, 0.125};
  GSTRIDE(c, mc) {
    const int I = (int)(c % mx), J = (int)((c / mx) % my), K = (int)(c / ((long long)mx * my));
    double f[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int c3 = 0; c3 < 5; ++c3) {
      const int k = (4 * K + c3 - 2 + nz) % nz;
      for (int b3 = 0; b3 < 5; ++b3) {
        const int j = (4 * J + b3 - 2 + ny) % ny;
        const double wbc = wt[b3] * wt[c3];
        for (int a3 = 0; a3 < 5; ++a3) {
          const int i = (4 * I + a3 - 2 + nx) % nx;
          const long long m = i + (long long)nx * (j + (long long)ny * k);
          const double w = wt[a3] * wbc;
          const double u = ux[m], v = uy[m], ww = uz[m];
          f[0] += w * u; f[1] += w * v; f[2] += w * ww;
          f[3] += w * u * u; f[4] += w * v * v; f[5] += w * ww * ww;
          f[6] += w * u * v; f[7] += w * u * ww; f[8] += w * v * ww;
        }
      }
    }
    o3.t[0][c] = f[0]; o3.t[1][c] = f[1]; o3.t[2][c] = f[2];
    o6.t[0][c] = f[3] - f[0] * f[0];
    o6.t[1][c] = f[4] - f[1] * f[1];
    o6.t[2][c] = f[5] - f[2] * f[2];
    o6.t[3][c] = f[6] - f[0] * f[1];
    o6.t[4][c] = f[7] - f[0] * f[2];
    o6.t[5][c] = f[8] - f[1] * f[2];
  }
}

}  // namespace

struct Mlp {
  float* P = nullptr;   // parameters
  float* m1 = nullptr;  // Adam moments
  float* m2 = nullptr;
  float* sc = nullptr;  // input scales (NI) | output scales (NO)
  float* part = nullptr;
  float* lpart = nullptr;
  float* lsum = nullptr;
  int nbmax = 0;
  int step = 0;
  float lam = 0.f, pscale = 1.f;  // energy-flux loss term
  // tensor-core inference (x3d_mlp_tc.cu): packed BF16 weight image, rebuilt
  // after every parameter change, and the device flag of its bounded waits
  bool tc = false;
  bool wp_dirty = true;
  void* wp = nullptr;
  int* tc_err = nullptr;
  ~Mlp() {
    for (float* p : {P, m1, m2, sc, part, lpart, lsum})
      if (p) cudaFree(p);
    if (wp) cudaFree(wp);
    if (tc_err) cudaFree(tc_err);
  }
};

// Packed weights for the tensor-core kernel, made on first use and after each
// parameter change (stream-ordered with the update that changed them).
static int tc_ready(Mlp* m, cudaStream_t st) {
  if (!m->wp) {
    if (cudaMalloc(&m->wp, MLP_TC_WP_BYTES) != cudaSuccess) return X3D_ERR_NOMEM;
    if (cudaMalloc(&m->tc_err, sizeof(int)) != cudaSuccess) return X3D_ERR_NOMEM;
    if (cudaMemsetAsync(m->tc_err, 0, sizeof(int), st) != cudaSuccess) return X3D_ERR_CUDA;
    m->wp_dirty = true;
  }
  if (m->wp_dirty) {
    const int rc = mlp_tc_pack(m->P, m->wp, st);
    if (rc != X3D_OK) return rc;
    m->wp_dirty = false;
  }
  return X3D_OK;
}

int mlp_les_tau(Mlp* m, const double* const* g9, double delta, double* const* tau6, long long n, int num_sms,
                cudaStream_t st) {
  if (m->tc) {
    const int rc = tc_ready(m, st);
    if (rc != X3D_OK) return rc;
    return mlp_tc_infer(m->P, m->sc, m->wp, m->tc_err, nullptr, nullptr, g9, (float)delta, tau6, n, num_sms, st);
  }
  G9 g;
  T6 t;
  for (int i = 0; i < 9; ++i) g.g[i] = g9[i];
  for (int i = 0; i < 6; ++i) t.t[i] = tau6[i];
  const size_t smem = (NPAR + NI + NO) * sizeof(float);
  k_mlp_les<<<num_sms * 4, 256, smem, st>>>(m->P, m->sc, g, (float)delta, t, n);
  return cuda_status(cudaGetLastError());
}

}  // namespace x3d

using namespace x3d;

extern "C" {

int x3d_mlp_create(int nin, int nhidden, int nout, x3d_mlp** out) {
  if (!out) return X3D_ERR_ARG;
  *out = nullptr;
  if (nin != NI || nhidden != NH || nout != NO) return X3D_ERR_UNSUPPORTED;
  Mlp* m = new Mlp();
  bool ok = cudaMalloc(&m->P, NPAR * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->m1, NPAR * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->m2, NPAR * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->sc, (NI + NO) * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->lsum, sizeof(float)) == cudaSuccess;
  if (!ok) {
    delete m;
    return X3D_ERR_NOMEM;
  }
  cudaMemset(m->P, 0, NPAR * sizeof(float));
  cudaMemset(m->m1, 0, NPAR * sizeof(float));
  cudaMemset(m->m2, 0, NPAR * sizeof(float));
  std::vector<float> one(NI + NO, 1.f);
  cudaMemcpy(m->sc, one.data(), one.size() * sizeof(float), cudaMemcpyHostToDevice);
  *out = reinterpret_cast<x3d_mlp*>(m);
  return cuda_status(cudaGetLastError());
}

int x3d_mlp_destroy(x3d_mlp* h) {
  delete reinterpret_cast<Mlp*>(h);
  return X3D_OK;
}

int x3d_mlp_param_count(void) { return NPAR; }

int x3d_mlp_set_params(x3d_mlp* h, const float* params, const float* scales) {
  if (!h) return X3D_ERR_ARG;
  Mlp* m = reinterpret_cast<Mlp*>(h);
  if (params && cudaMemcpy(m->P, params, NPAR * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return X3D_ERR_CUDA;
  if (scales && cudaMemcpy(m->sc, scales, (NI + NO) * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return X3D_ERR_CUDA;
  m->step = 0;
  m->wp_dirty = true;
  cudaMemset(m->m1, 0, NPAR * sizeof(float));
  cudaMemset(m->m2, 0, NPAR * sizeof(float));
  return cuda_status(cudaGetLastError());
}

int x3d_mlp_get_params(x3d_mlp* h, float* params, float* scales) {
  if (!h) return X3D_ERR_ARG;
  Mlp* m = reinterpret_cast<Mlp*>(h);
  if (params && cudaMemcpy(params, m->P, NPAR * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return X3D_ERR_CUDA;
  if (scales && cudaMemcpy(scales, m->sc, (NI + NO) * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return X3D_ERR_CUDA;
  return X3D_OK;
}

int x3d_mlp_infer(x3d_mlp* h, const float* X, float* Y, long long n, void* stream) {
  if (!h || !X || !Y || n < 0) return X3D_ERR_ARG;
  Mlp* m = reinterpret_cast<Mlp*>(h);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (m->tc) {
    const int rc = tc_ready(m, (cudaStream_t)stream);
    if (rc != X3D_OK) return rc;
    return mlp_tc_infer(m->P, m->sc, m->wp, m->tc_err, X, Y, nullptr, 0.f, nullptr, n, sms, (cudaStream_t)stream);
  }
  const size_t smem = (NPAR + NI + NO) * sizeof(float);
  k_mlp_infer<<<sms * 4, 256, smem, (cudaStream_t)stream>>>(m->P, m->sc, X, Y, n);
  return cuda_status(cudaGetLastError());
}

int x3d_mlp_train_step(x3d_mlp* h, const float* X, const float* T, long long n, float lr, float* loss,
                       void* stream) {
  if (!h || !X || !T || n <= 0) return X3D_ERR_ARG;
  Mlp* m = reinterpret_cast<Mlp*>(h);
  cudaStream_t st = (cudaStream_t)stream;
  const long long nbl = (n + TB - 1) / TB;
  if (nbl > (1 << 20)) return X3D_ERR_ARG;
  const int nb = (int)nbl;
  if (nb > m->nbmax) {
    if (m->part) cudaFree(m->part);
    if (m->lpart) cudaFree(m->lpart);
    m->part = m->lpart = nullptr;
    if (cudaMalloc(&m->part, (size_t)nb * NPAR * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->lpart, (size_t)nb * sizeof(float)) != cudaSuccess)
      return X3D_ERR_NOMEM;
    m->nbmax = nb;
  }
  const size_t smem = (NPAR + NI + NO + (NI + 4 * NH + NO) * PD + TB) * sizeof(float);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    configured = true;
  }
  k_mlp_grad<<<nb, TB, smem, st>>>(m->P, m->sc, X, T, n, m->lam, m->pscale, m->part, m->lpart);
  m->step += 1;
  const float b1c = 1.f - powf(0.9f, (float)m->step), b2c = 1.f - powf(0.999f, (float)m->step);
  k_mlp_adam<<<(NPAR + 255) / 256, 256, 0, st>>>(m->P, m->m1, m->m2, m->part, nb, lr, b1c, b2c);
  m->wp_dirty = true;
  if (loss) {
    k_sum<<<1, 1, 0, st>>>(m->lpart, nb, m->lsum);
    float hl = 0.f;
    if (cudaMemcpyAsync(&hl, m->lsum, sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess) return X3D_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return X3D_ERR_CUDA;
    *loss = hl / (float)n;
  }
  return cuda_status(cudaGetLastError());
}

int x3d_mlp_set_tensor_cores(x3d_mlp* h, int on) {
  if (!h || (on != 0 && on != 1)) return X3D_ERR_ARG;
  Mlp* m = reinterpret_cast<Mlp*>(h);
  m->tc = on != 0;
  return X3D_OK;
}

int x3d_mlp_status(x3d_mlp* h) {
  if (!h) return X3D_ERR_ARG;
  Mlp* m = reinterpret_cast<Mlp*>(h);
  if (!m->tc_err) return X3D_OK;
  int e = 0;
  // inference may run on any stream, blocking or not: wait for all of them
  if (cudaDeviceSynchronize() != cudaSuccess) return X3D_ERR_CUDA;
  if (cudaMemcpy(&e, m->tc_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return X3D_ERR_CUDA;
  return e ? X3D_ERR_CUDA : X3D_OK;
}

int x3d_mlp_set_flux_loss(x3d_mlp* h, float lam, float pscale) {
  if (!h || !(pscale > 0.f) || lam < 0.f) return X3D_ERR_ARG;
  Mlp* m = reinterpret_cast<Mlp*>(h);
  m->lam = lam;
  m->pscale = pscale;
  return X3D_OK;
}

int x3d_box_filter4(const double* ux, const double* uy, const double* uz, int nx, int ny, int nz, double* ubar,
                    double* vbar, double* wbar, double* tau, void* stream) {
  if (!ux || !uy || !uz || !ubar || !vbar || !wbar || !tau) return X3D_ERR_ARG;
  if (nx % 4 || ny % 4 || nz % 4 || nx < 8 || ny < 8 || nz < 8) return X3D_ERR_SHAPE;
  const long long mc = (long long)(nx / 4) * (ny / 4) * (nz / 4);
  T6 o3, o6;
  o3.t[0] = ubar; o3.t[1] = vbar; o3.t[2] = wbar;
  for (int q = 0; q < 6; ++q) o6.t[q] = tau + (size_t)q * mc;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_box4_stress<<<sms * 8, 256, 0, (cudaStream_t)stream>>>(ux, uy, uz, nx, ny, nz, o3, o6);
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
