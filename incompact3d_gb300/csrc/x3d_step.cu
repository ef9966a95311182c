// Incompressible time step for the plain periodic case, resident in HBM:
//   calculate_transeq_rhs -> intt -> divergence -> poisson -> gradp -> cor_vel
// (src/xcompact3d.f90:29-102, src/transeq.f90:73-591,
//  src/time_integrators.f90:18-187, src/navier.f90:27-499), plus the TGV
// statistics of postprocess_tgv (src/Case-TGV.f90:189-477).
//
// The 2DECOMP transposes between stages are identities on one GPU (X-, Y- and
// Z-pencils are the same (nx,ny,nz) array), so the stages read the x-pencil
// fields directly.  Time-integrator history is rotated by pointer, never copied.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "x3d_df.cuh"
#include "x3d_internal.h"

namespace x3d {

// ---------------------------------------------------------------------------
// Pointwise kernels (grid-stride, 3 components per thread)
// ---------------------------------------------------------------------------
namespace {

inline unsigned pw_blocks(Ctx* c, long long n) {
  const long long per = 256LL * 4;
  long long b = (n + per - 1) / per;
  const long long cap = (long long)c->num_sms * 8;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

#define GRID_STRIDE(i, n) \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

// Adams-Bashforth / RK update, FP64 operators:
//   u = c1*h1 + c2*h2 + c3*h3 + u   (nh = number of history terms used)
__global__ void k_intt64(double* u, const double* h1, const double* h2, const double* h3, double c1, double c2,
                         double c3, int nh, long long n) {
  GRID_STRIDE(i, n) {
    double acc = c1 * h1[i];
    if (nh > 1) acc = acc + c2 * h2[i];
    if (nh > 2) acc = acc + c3 * h3[i];
    u[i] = acc + u[i];
  }
}


// AB/RK update of the double-float state: (h,l) += sum(c_k h_k), the increment
// formed in FP32 (it carries the FP32 accuracy of the right-hand sides).
struct Intt3 {
  float* uh[3];
  float* ul[3];
  const float* h[3][3];
};
__global__ void k_intt_df(Intt3 a, float c1, float c2, float c3, int nh, long long n) {
  GRID_STRIDE(i, n) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      float inc = c1 * a.h[q][0][i];
      if (nh > 1) inc = inc + c2 * a.h[q][1][i];
      if (nh > 2) inc = inc + c3 * a.h[q][2][i];
      float h = a.uh[q][i], l = a.ul[q][i];
      df_add_f(h, l, inc);
      a.uh[q][i] = h;
      a.ul[q][i] = l;
    }
  }
}

// The same update on 4 consecutive points per thread with 16-byte accesses
// (n a multiple of 4, 16-byte aligned fields): fewer instructions per byte.
__device__ __forceinline__ float f4get(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
__device__ __forceinline__ void f4set(float4& v, int k, float x) {
  if (k == 0) v.x = x; else if (k == 1) v.y = x; else if (k == 2) v.z = x; else v.w = x;
}
__global__ void k_intt_df4(Intt3 a, float c1, float c2, float c3, int nh, long long n4) {
  GRID_STRIDE(i, n4) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float4 h0 = reinterpret_cast<const float4*>(a.h[q][0])[i];
      const float4 h1 = nh > 1 ? reinterpret_cast<const float4*>(a.h[q][1])[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 h2 = nh > 2 ? reinterpret_cast<const float4*>(a.h[q][2])[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      float4 uh = reinterpret_cast<const float4*>(a.uh[q])[i];
      float4 ul = reinterpret_cast<const float4*>(a.ul[q])[i];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        float inc = c1 * f4get(h0, k);
        if (nh > 1) inc = inc + c2 * f4get(h1, k);
        if (nh > 2) inc = inc + c3 * f4get(h2, k);
        float h = f4get(uh, k), l = f4get(ul, k);
        df_add_f(h, l, inc);
        f4set(uh, k, h);
        f4set(ul, k, l);
      }
      reinterpret_cast<float4*>(a.uh[q])[i] = uh;
      reinterpret_cast<float4*>(a.ul[q])[i] = ul;
    }
  }
}

// cor_vel on the double-float state: u -= grad p (FP32 gradient)
struct Cor3 {
  float* uh[3];
  float* ul[3];
  const float* p[3];
};
__global__ void k_corvel_df(Cor3 a, long long n) {
  GRID_STRIDE(i, n) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      float h = a.uh[q][i], l = a.ul[q][i];
      df_add_f(h, l, -a.p[q][i]);
      a.uh[q][i] = h;
      a.ul[q][i] = l;
    }
  }
}

__global__ void k_corvel_df4(Cor3 a, long long n4) {
  GRID_STRIDE(i, n4) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float4 p = reinterpret_cast<const float4*>(a.p[q])[i];
      float4 uh = reinterpret_cast<const float4*>(a.uh[q])[i];
      float4 ul = reinterpret_cast<const float4*>(a.ul[q])[i];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        float h = f4get(uh, k), l = f4get(ul, k);
        df_add_f(h, l, -f4get(p, k));
        f4set(uh, k, h);
        f4set(ul, k, l);
      }
      reinterpret_cast<float4*>(a.uh[q])[i] = uh;
      reinterpret_cast<float4*>(a.ul[q])[i] = ul;
    }
  }
}

__global__ void k_split(float* h, float* l, const double* d, long long n) {
  GRID_STRIDE(i, n) {
    const double v = d[i];
    const float hi = (float)v;
    h[i] = hi;
    l[i] = (float)(v - (double)hi);
  }
}

__global__ void k_combine(double* d, const float* h, const float* l, long long n) {
  GRID_STRIDE(i, n) d[i] = (double)h[i] + (double)l[i];
}

template <typename T>
__global__ void k_add(T* o, const T* a, const T* b, long long n) {
  GRID_STRIDE(i, n) o[i] = a[i] + b[i];
}

template <typename T>
__global__ void k_add_to64(double* o, const T* a, const T* b, long long n) {
  GRID_STRIDE(i, n) o[i] = (double)(a[i] + b[i]);
}

__global__ void k_to32(float* o, const double* a, long long n) {
  GRID_STRIDE(i, n) o[i] = (float)a[i];
}

// u -= px (cor_vel), FP64 state
template <typename T>
__global__ void k_corvel(double* u1, double* u2, double* u3, const T* p1, const T* p2, const T* p3, long long n) {
  GRID_STRIDE(i, n) {
    u1[i] = u1[i] - (double)p1[i];
    u2[i] = u2[i] - (double)p2[i];
    u3[i] = u3[i] - (double)p3[i];
  }
}

__global__ void k_tgv_init(double* ux, double* uy, double* uz, int nx, int ny, int nz, double dx, double dy,
                           double dz) {
  const long long n = (long long)nx * ny * nz;
  GRID_STRIDE(m, n) {
    const int i = (int)(m % nx);
    const int j = (int)((m / nx) % ny);
    const int k = (int)(m / ((long long)nx * ny));
    const double x = (double)i * dx, y = (double)j * dy, z = (double)k * dz;
    ux[m] = sin(x) * cos(y) * cos(z);
    uy[m] = -cos(x) * sin(y) * cos(z);
    uz[m] = 0.0;
  }
}

// Block partial sums for the TGV statistics; one value per block per quantity.
// q: 0 = 0.5*sum(u^2+v^2+w^2); 1 = eps(strain); 2 = enstrophy; 3 = eps2
// Sums of postprocess_tgv over the points i < sx, j < sy, k < sz (the last
// point of a free-slip axis is left out, src/Case-TGV.f90:211-226).
__global__ void k_stats(const double* ux, const double* uy, const double* uz, const double* const* g,
                        const double* const* l, double xnu, long long n, int nx, int ny, int sx, int sy, int sz,
                        double* part) {
  __shared__ double sh[4][256];
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  GRID_STRIDE(m, n) {
    const long long pl = (long long)nx * ny;
    const int k = (int)(m / pl), j = (int)((m - (long long)k * pl) / nx), i = (int)(m - (long long)k * pl - (long long)j * nx);
    if (i >= sx || j >= sy || k >= sz) continue;
    const double u = ux[m], v = uy[m], w = uz[m];
    a0 += 0.5 * (u * u + v * v + w * w);
    // g: 0 du/dx 1 dv/dx 2 dw/dx 3 du/dy 4 dv/dy 5 dw/dy 6 du/dz 7 dv/dz 8 dw/dz
    const double ta = g[0][m], tb = g[1][m], tc = g[2][m], td = g[3][m], te = g[4][m], tf = g[5][m], tg = g[6][m],
                 th = g[7][m], ti = g[8][m];
    const double s1 = 2.0 * ta, s2 = 2.0 * te, s3 = 2.0 * ti, s4 = td + tb, s5 = tg + tc, s6 = th + tf;
    a1 += 0.5 * xnu * (s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4) + 2.0 * (s5 * s5) + 2.0 * (s6 * s6));
    const double o1 = tf - th, o2 = tg - tc, o3 = tb - td;
    a2 += 0.5 * (o1 * o1 + o2 * o2 + o3 * o3);
    a3 += (-xnu) * (u * (l[0][m] + l[3][m] + l[6][m]) + v * (l[1][m] + l[4][m] + l[7][m]) +
                    w * (l[2][m] + l[5][m] + l[8][m]));
  }
  sh[0][threadIdx.x] = a0; sh[1][threadIdx.x] = a1; sh[2][threadIdx.x] = a2; sh[3][threadIdx.x] = a3;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 4) part[(size_t)blockIdx.x * 4 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_absmax(const double* a, long long n, double* part) {
  __shared__ double sh[256];
  double m = 0;
  GRID_STRIDE(i, n) m = fmax(m, fabs(a[i]));
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

}  // namespace

// ---- channel case (walls at y = 0 and y = Ly, x and z periodic) -------------
// channel_cfr (src/Case-Channel.f90:221-264): block partial sums of u/ppy(j).
__global__ void k_cfr_partial(const double* ux, const double* ppy, int nx, int ny, long long n, double* part) {
  __shared__ double sh[256];
  double acc = 0.0;
  GRID_STRIDE(m, n) {
    const int j = (int)((m / nx) % ny);
    acc += ux[m] / ppy[j];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
// ub = sum * coeff; can = -(target - ub); ub and can go to out[0], out[1].
__global__ void k_cfr_finish(const double* part, int nparts, double coeff, double target, double* out) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nparts; b += 256) acc += part[b];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double ub = sh[0] * coeff;
    out[0] = ub;
    out[1] = -(target - ub);
  }
}
__global__ void k_sub_dev(double* u, const double* c, long long n) {
  const double v = *c;
  GRID_STRIDE(i, n) u[i] = u[i] - v;
}
// momentum_forcing_channel rotation (src/Case-Channel.f90:413-418)
__global__ void k_rotation(double* hx, double* hy, const double* ux, const double* uy, double w, long long n) {
  GRID_STRIDE(i, n) {
    const double a = hx[i] - w * uy[i];
    const double b = hy[i] + w * ux[i];
    hx[i] = a;
    hy[i] = b;
  }
}
// Stretched-mesh y-viscous term folded into the running sum
// (src/transeq.f90:335-370 and 426-430):
//   tz = xnu * (dyy * pp2y(j) - pp4y(j) * dy) + (tz - th/2)
__global__ void k_visc_y_stretch(double* tz, const double* dyy, const double* dy, const double* th,
                                 const double* pp2y, const double* pp4y, double xnu, int nx, int ny, long long n) {
  GRID_STRIDE(m, n) {
    const int j = (int)((m / nx) % ny);
    const double td = dyy[m] * pp2y[j] - pp4y[j] * dy[m];
    tz[m] = xnu * td + (tz[m] - 0.5 * th[m]);
  }
}
// pre_correc no-slip walls (src/navier.f90:614-700): the stored tangential
// pressure gradients are rescaled by gdt and imposed as the wall velocity.
__global__ void k_walls(double* ux, double* uy, double* uz, double* dp, double g, int nx, int ny, int nz) {
  const long long nw = (long long)nx * nz;
  double* dpdx1 = dp;
  double* dpdz1 = dp + nw;
  double* dpdxn = dp + 2 * nw;
  double* dpdzn = dp + 3 * nw;
  GRID_STRIDE(w, nw) {
    const long long i = w % nx, k = w / nx;
    dpdx1[w] = dpdx1[w] * g;
    dpdz1[w] = dpdz1[w] * g;
    dpdxn[w] = dpdxn[w] * g;
    dpdzn[w] = dpdzn[w] * g;
    const long long b = i + (long long)nx * ny * k, t = b + (long long)nx * (ny - 1);
    ux[b] = 0.0 + dpdx1[w];
    uy[b] = 0.0;
    uz[b] = 0.0 + dpdz1[w];
    ux[t] = 0.0 + dpdxn[w];
    uy[t] = 0.0;
    uz[t] = 0.0 + dpdzn[w];
  }
}
// gradp's wall-gradient storage (src/navier.f90:456-477)
__global__ void k_wallgrad(double* dp, const double* px, const double* pz, double g, int nx, int ny, int nz) {
  const long long nw = (long long)nx * nz;
  GRID_STRIDE(w, nw) {
    const long long i = w % nx, k = w / nx;
    const long long b = i + (long long)nx * ny * k, t = b + (long long)nx * (ny - 1);
    dp[w] = px[b] / g;
    dp[nw + w] = pz[b] / g;
    dp[2 * nw + w] = px[t] / g;
    dp[3 * nw + w] = pz[t] / g;
  }
}

// ---- explicit LES (src/les_models.f90) -----------------------------------
__global__ void k_les_prod(double* p0, double* p1, double* p2, double* p3, double* p4, double* p5,
                           const double* ux, const double* uy, const double* uz, long long n) {
  GRID_STRIDE(m, n) {
    const double a = ux[m], b = uy[m], c = uz[m];
    p0[m] = a * a; p1[m] = b * b; p2[m] = c * c;
    p3[m] = a * b; p4[m] = a * c; p5[m] = b * c;
  }
}
struct Six {
  double* v[6];
};
struct CSix {
  const double* v[6];
};
// srt = S:S (smag, src/les_models.f90:265-267)
__global__ void k_les_srt(double* srt, CSix S, long long n) {
  GRID_STRIDE(m, n) {
    const double xx = S.v[0][m], yy = S.v[1][m], zz = S.v[2][m], xy = S.v[3][m], xz = S.v[4][m], yz = S.v[5][m];
    srt[m] = xx * xx + yy * yy + zz * zz + 2.0 * xy * xy + 2.0 * xz * xz + 2.0 * yz * yz;
  }
}
// out_q = -2 sqrt(2 S:S) S_q * (f del(j))^2 (dynsmag's a_ij with f = 1 and
// b_ij with f = 2, src/les_models.f90:609-676); out may alias S.
__global__ void k_les_tensor(Six out, CSix S, const double* del, double f, int nx, int ny, long long n) {
  GRID_STRIDE(m, n) {
    const double xx = S.v[0][m], yy = S.v[1][m], zz = S.v[2][m], xy = S.v[3][m], xz = S.v[4][m], yz = S.v[5][m];
    const double mag = sqrt(2.0 * (xx * xx + yy * yy + zz * zz + 2.0 * xy * xy + 2.0 * xz * xz + 2.0 * yz * yz));
    const double dl = f * del[(m / nx) % ny];
    const double d2 = dl * dl;
    const double s6[6] = {xx, yy, zz, xy, xz, yz};
#pragma unroll
    for (int q = 0; q < 6; ++q) out.v[q][m] = (-2.0 * mag * s6[q]) * d2;
  }
}
// L_ij = (u_i u_j)^f - u_i^f u_j^f, in place on the filtered products
__global__ void k_les_leonard(Six P, const double* uf, const double* vf, const double* wf, long long n) {
  GRID_STRIDE(m, n) {
    const double a = uf[m], b = vf[m], c = wf[m];
    P.v[0][m] = P.v[0][m] - a * a;
    P.v[1][m] = P.v[1][m] - b * b;
    P.v[2][m] = P.v[2][m] - c * c;
    P.v[3][m] = P.v[3][m] - a * b;
    P.v[4][m] = P.v[4][m] - a * c;
    P.v[5][m] = P.v[5][m] - b * c;
  }
}
// dynamic constant (src/les_models.f90:780-811): M = b - a^f, deviatoric L
// (statement by statement as written), C = L:M / M:M clipped to [0, cmax]
__global__ void k_les_smagc(double* C, CSix L, CSix B, CSix A, double cmax, long long n) {
  GRID_STRIDE(m, n) {
    const double mxx = B.v[0][m] - A.v[0][m], myy = B.v[1][m] - A.v[1][m], mzz = B.v[2][m] - A.v[2][m];
    const double mxy = B.v[3][m] - A.v[3][m], mxz = B.v[4][m] - A.v[4][m], myz = B.v[5][m] - A.v[5][m];
    double lxx = L.v[0][m], lyy = L.v[1][m], lzz = L.v[2][m];
    const double lxy = L.v[3][m], lxz = L.v[4][m], lyz = L.v[5][m];
    lxx = lxx - (lxx + lyy + lzz) / 3.0;
    lyy = lyy - (lxx + lyy + lzz) / 3.0;
    lzz = lzz - (lxx + lyy + lzz) / 3.0;
    double v = (lxx * mxx + lyy * myy + lzz * mzz + 2.0 * (lxy * mxy + lxz * mxz + lyz * myz)) /
               (mxx * mxx + myy * myy + mzz * mzz + 2.0 * (mxy * mxy + mxz * mxz + myz * myz));
    if (v > cmax) v = cmax;
    if (v < 0.0) v = 0.0;
    C[m] = v;
  }
}
// nut = <C>_z del(j)^2 sqrt(2 srt): mean over z per (x, y) column
// (mean_plane_z, src/tools.f90:982-996), summed in k order
__global__ void k_les_nut_dyn(double* nut, const double* cf, const double* srt, const double* del, int nx, int ny,
                              int nz) {
  const long long ncol = (long long)nx * ny;
  GRID_STRIDE(col, ncol) {
    const long long plane = ncol;
    double sum = 0.0;
    for (int k = 0; k < nz; ++k) sum = sum + cf[col + k * plane];
    const double cm = sum / (double)nz;
    const double dl = del[col / nx];
    for (int k = 0; k < nz; ++k) {
      const long long m = col + k * plane;
      nut[m] = cm * (dl * dl) * sqrt(2.0 * srt[m]);
    }
  }
}
// smag: nut = (Cs del(j))^2 sqrt(2 srt)
__global__ void k_les_nut_smag(double* nut, const double* srt, const double* del, double cs, int nx, int ny,
                               long long n) {
  GRID_STRIDE(m, n) {
    const double length = cs * del[(m / nx) % ny];
    nut[m] = (length * length) * sqrt(2.0 * srt[m]);
  }
}
// sgs_mom_nonconservative terms of one direction (src/les_models.f90:1115-1232):
//   g_q (+)= nut * d2_q + 2 S_q * dnut      (first = 1: assignment)
__global__ void k_les_sgs(double* gx, double* gy, double* gz, const double* d2x, const double* d2y,
                          const double* d2z, const double* nut, const double* dnut, const double* sa,
                          const double* sb, const double* sc, int first, long long n) {
  GRID_STRIDE(m, n) {
    const double nu = nut[m], dn = dnut[m];
    if (first) {
      gx[m] = d2x[m] * nu + 2.0 * sa[m] * dn;
      gy[m] = d2y[m] * nu + 2.0 * sb[m] * dn;
      gz[m] = d2z[m] * nu + 2.0 * sc[m] * dn;
    } else {
      gx[m] = gx[m] + nu * d2x[m] + 2.0 * sa[m] * dn;
      gy[m] = gy[m] + nu * d2y[m] + 2.0 * sb[m] * dn;
      gz[m] = gz[m] + nu * d2z[m] + 2.0 * sc[m] * dn;
    }
  }
}
// stretched-mesh second derivative: t = t pp2y(j) - pp4y(j) dy
__global__ void k_stretch_d2(double* t, const double* dy, const double* pp2y, const double* pp4y, int nx, int ny,
                             long long n) {
  GRID_STRIDE(m, n) {
    const int j = (int)((m / nx) % ny);
    t[m] = t[m] * pp2y[j] - pp4y[j] * dy[m];
  }
}
__global__ void k_add3(double* hx, double* hy, double* hz, const double* gx, const double* gy, const double* gz,
                       long long n) {
  GRID_STRIDE(m, n) {
    hx[m] = hx[m] + gx[m];
    hy[m] = hy[m] + gy[m];
    hz[m] = hz[m] + gz[m];
  }
}

// ---------------------------------------------------------------------------
// Solver
// ---------------------------------------------------------------------------
struct SolverImpl {
  Ctx* c = nullptr;
  x3d_solver_opts o;
  long long N = 0, Np = 0;  // velocity-mesh and pressure-mesh sizes
  int itime = 0;            // completed steps
  int ntime = 3, nsub = 1;
  double adt[3] = {0, 0, 0}, bdt[3] = {0, 0, 0}, cdt[3] = {0, 0, 0}, gdt[3] = {0, 0, 0};
  // FP64 state (FP64 mode); staging for set/get/statistics (mixed mode)
  double *ux = nullptr, *uy = nullptr, *uz = nullptr;
  // mixed mode: double-float state (hi, lo); hi is the operators' FP32 input
  float* uh[3] = {nullptr, nullptr, nullptr};
  float* ul[3] = {nullptr, nullptr, nullptr};
  // history: [component][slot], precision of the operators
  void* H[3][3] = {{nullptr}};
  // work fields in operator precision
  void* W[16] = {nullptr};
  void* P[8] = {nullptr};  // pressure-mesh / intermediate-mesh work
  double* pp64 = nullptr;    // pressure (FP64 solvers)
  float* p32 = nullptr;      // pressure of the mixed-precision solver (binary32)
  double* part = nullptr;  // reduction partials
  double* hpart = nullptr;
  int launches = 0;
  // channel case: walls in y (x, z periodic)
  bool walls = false;       // geometry: y non-periodic with ncl 2/2
  bool slip = false;        // geometry: free-slip x and y, z free-slip or periodic (poisson_11x)
  bool cfr = false;         // constant flow rate control (channel_cfr)
  double cfr_target = 2.0 / 3.0, wrotation = 0.0;
  int spinup_time = 0;
  double* wall_dp = nullptr;  // dpdxy1 | dpdzy1 | dpdxyn | dpdzyn (nx*nz each)
  double* ub_dev = nullptr;   // per sub-step: ub, can (2 x nsub)
  // explicit LES (FP64): jles 1 Smagorinsky, 3 dynamic Smagorinsky
  int jles = 0;
  double smagcst = 0.14, maxdsmagcst = 0.3;
  double* del = nullptr;      // filter width per y row (device, ny)
  x3d_ctx* cf = nullptr;      // context whose filter has alpha = 0 (dynsmag's filter(zero))
  double* lw[40] = {nullptr}; // LES work fields
  Mlp* mlp = nullptr;         // learned closure (jles = 10), not owned
  std::vector<void*> allocs;
  // asynchronous host transfers: a read-out stream (xs[0]) and a write-in
  // stream (xs[1]); per-component events order a component's write-in after
  // its read-out, and the steps around them
  bool xfer_init = false;
  cudaStream_t xs[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_set[3] = {nullptr, nullptr, nullptr}, ev_get[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_step = nullptr;
  ~SolverImpl() {
    if (xfer_init) {
      for (int q = 0; q < 3; ++q) {
        cudaStreamSynchronize(xs[q]);
        cudaStreamDestroy(xs[q]);
        cudaEventDestroy(ev_set[q]);
        cudaEventDestroy(ev_get[q]);
      }
      cudaEventDestroy(ev_step);
    }
    for (void* p : allocs) cudaFree(p);
    if (hpart) cudaFreeHost(hpart);
    if (cf) x3d_ctx_destroy(cf);
  }
  template <typename T>
  T* alloc(long long n) {
    void* p = nullptr;
    if (cudaMalloc(&p, (size_t)n * sizeof(T)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (T*)p;
  }
  bool mixed() const { return o.precision == X3D_PREC_MIXED; }
};

}  // namespace x3d

struct x3d_solver {
  x3d::SolverImpl impl;
};

namespace x3d {

template <typename T>
static int op(SolverImpl* s, int axis, int kind, int npaire, T* out, const T* in, const int* dims, cudaStream_t st,
              const Fuse<T>* fz = nullptr, const T* pp = nullptr) {
  OpPlan* p = nullptr;
  int rc = get_plan(s->c, axis, kind, npaire, default_coefset(kind, npaire), &p);
  if (rc != X3D_OK) return rc;
  s->launches++;
  return launch_line_op<T>(s->c, p, out, in, dims, pp, st, fz);
}

// y metric of a stretched mesh for operators in precision T (FP64 only):
// which 0 = ppy, 1 = pp2y, 2 = pp4y, 3 = ppyi; null on a uniform mesh.
template <typename T>
static const T* ymetric(SolverImpl* s, int which) {
  if (s->c->st.istret == 0 || !std::is_same<T, double>::value) return nullptr;
  const double* d = nullptr;
  if (stretch_device(s->c, &d) != X3D_OK) return nullptr;
  return reinterpret_cast<const T*>(d + (size_t)which * s->c->grid.ny);
}

template <typename T>
Fuse<T> fz_prod(const T* in2) {
  Fuse<T> f;
  f.in2 = in2;
  return f;
}
template <typename T>
Fuse<T> fz_comb(T cr, const T* a1, T c1, const T* a2, T c2, const T* y) {
  Fuse<T> f;
  f.cr = cr; f.a1 = a1; f.c1 = c1; f.a2 = a2; f.c2 = c2; f.y = y;
  f.active = 1;
  return f;
}

#define RC(x)                      \
  do {                             \
    int _r = (x);                  \
    if (_r != X3D_OK) return _r;   \
  } while (0)

// momentum_rhs_eq (src/transeq.f90:73-591) for the incompressible periodic
// case, in operator precision T.  For each component u_q and direction j the
// reference forms conv_j = d_j(u_q u_j) + u_j d_j u_q and nu d_jj u_q between
// transposes; here every product is formed while a line kernel loads its
// input and every sum while it stores its output, so the 27 line solves carry
// all the pointwise work and no separate elementwise pass touches HBM:
//   X: t1 = dx(ux*uq);   tg = t1 + ux*dx(uq)
//   Y: t1 = dy(uy*uq);   th = t1 + uy*dy(uq)
//   Z: t1 = dz(uz*uq);   tz = t1 + uz*dz(uq);   tz = nu*dzz(uq) - tz/2
//   Y: tz = nu*dyy(uq) + tz - th/2
//   X: H_q = nu*dxx(uq) + tz - tg/2
// Parities follow the reference's calls: npaire = 0 for d_j u_j and d_jj u_j,
// 1 for the other components (and the reverse for the products).
template <typename T>
static int momentum_rhs(SolverImpl* s, const T* const* u, T* const* H, cudaStream_t st) {
  Ctx* c = s->c;
  const int dims[3] = {c->grid.nx, c->grid.ny, c->grid.nz};
  T** w = reinterpret_cast<T**>(s->W);
  T *t1 = w[0], *tg = w[1], *th = w[2], *tz = w[3];
  const T xnu = (T)s->o.xnu;
  const T one = T(1), mhalf = T(-0.5), zero = T(0);
  // stretched mesh: dery multiplies by ppy; d2/dy2 gets the pp2y / pp4y terms
  const T* ppy = ymetric<T>(s, 0);
  if (std::is_same<T, float>::value && !ppy && rhs_axis_fast_ok(c, 1, dims) && rhs_axis_fast_ok(c, 2, dims)) {
    // FP32 periodic lines: one fused kernel per axis runs the three solves of
    // a line (Z, then Y, then X into the history slot)
    for (int q = 0; q < 3; ++q) {
      const int pu[3] = {q == 0 ? 0 : 1, q == 1 ? 0 : 1, q == 2 ? 0 : 1};
      OpPlan* P[3][3];
      for (int ax = 0; ax < 3; ++ax) {
        RC(get_plan(c, ax, K_DER1, 1 - pu[ax], default_coefset(K_DER1, 1 - pu[ax]), &P[ax][0]));
        RC(get_plan(c, ax, K_DER1, pu[ax], default_coefset(K_DER1, pu[ax]), &P[ax][1]));
        RC(get_plan(c, ax, K_DER2, pu[ax], default_coefset(K_DER2, pu[ax]), &P[ax][2]));
      }
      float* tzf = (float*)tz;
      const float* uf[3] = {(const float*)u[0], (const float*)u[1], (const float*)u[2]};
      const float* uqf = uf[q];
      RC(rhs_axis_fast(c, P[2][0], P[2][1], P[2][2], tzf, uf[2], uqf, nullptr, (float)xnu, dims, st));
      RC(rhs_axis_fast(c, P[1][0], P[1][1], P[1][2], tzf, uf[1], uqf, tzf, (float)xnu, dims, st));
      s->launches += 2;
      if (rhs_axis_fast_ok(c, 0, dims)) {
        RC(rhs_axis_fast(c, P[0][0], P[0][1], P[0][2], (float*)H[q], uf[0], uqf, tzf, (float)xnu, dims, st));
        s->launches++;
      } else {
        Fuse<T> f = fz_prod<T>(u[q]);
        RC(op<T>(s, 0, K_DER1, 1 - pu[0], t1, u[0], dims, st, &f));
        f = fz_comb<T>(zero, t1, one, nullptr, zero, u[0]);
        RC(op<T>(s, 0, K_DER1, pu[0], tg, u[q], dims, st, &f));
        f = fz_comb<T>(xnu, tz, one, tg, mhalf, nullptr);
        RC(op<T>(s, 0, K_DER2, pu[0], H[q], u[q], dims, st, &f));
      }
    }
    return cuda_status(cudaGetLastError());
  }
  for (int q = 0; q < 3; ++q) {
    const T* uq = u[q];
    const int pu[3] = {q == 0 ? 0 : 1, q == 1 ? 0 : 1, q == 2 ? 0 : 1};  // parity of d_j u_q
    Fuse<T> f;
    // X
    f = fz_prod<T>(uq);
    RC(op<T>(s, 0, K_DER1, 1 - pu[0], t1, u[0], dims, st, &f));
    f = fz_comb<T>(zero, t1, one, nullptr, zero, u[0]);
    RC(op<T>(s, 0, K_DER1, pu[0], tg, uq, dims, st, &f));
    // Y
    f = fz_prod<T>(uq);
    RC(op<T>(s, 1, K_DER1, 1 - pu[1], t1, u[1], dims, st, &f, ppy));
    f = fz_comb<T>(zero, t1, one, nullptr, zero, u[1]);
    RC(op<T>(s, 1, K_DER1, pu[1], th, uq, dims, st, &f, ppy));
    // Z
    f = fz_prod<T>(uq);
    RC(op<T>(s, 2, K_DER1, 1 - pu[2], t1, u[2], dims, st, &f));
    f = fz_comb<T>(zero, t1, one, nullptr, zero, u[2]);
    RC(op<T>(s, 2, K_DER1, pu[2], tz, uq, dims, st, &f));
    f = fz_comb<T>(xnu, tz, mhalf, nullptr, zero, nullptr);
    RC(op<T>(s, 2, K_DER2, pu[2], tz, uq, dims, st, &f));
    // back to Y
    if (ppy) {
      T *tdy = w[5], *tdd = w[6];
      RC(op<T>(s, 1, K_DER1, pu[1], tdy, uq, dims, st, nullptr, ppy));
      RC(op<T>(s, 1, K_DER2, pu[1], tdd, uq, dims, st));
      const long long N = s->N;
      k_visc_y_stretch<<<pw_blocks(c, N), 256, 0, st>>>((double*)tz, (const double*)tdd, (const double*)tdy,
                                                        (const double*)th, (const double*)ymetric<T>(s, 1),
                                                        (const double*)ymetric<T>(s, 2), s->o.xnu, c->grid.nx,
                                                        c->grid.ny, N);
      s->launches++;
    } else {
      f = fz_comb<T>(xnu, tz, one, th, mhalf, nullptr);
      RC(op<T>(s, 1, K_DER2, pu[1], tz, uq, dims, st, &f));
    }
    // back to X: final sum into the history slot
    f = fz_comb<T>(xnu, tz, one, tg, mhalf, nullptr);
    RC(op<T>(s, 0, K_DER2, pu[0], H[q], uq, dims, st, &f));
  }
  return cuda_status(cudaGetLastError());
}

// divergence (nlock=1) of src/navier.f90:257-372: pp64 = div(u) on the
// pressure mesh, computed in T, written in FP64 for the Poisson solve.
template <typename T>
static int divergence(SolverImpl* s, const T* ux, const T* uy, const T* uz, void* pout, bool out64,
                      cudaStream_t st) {
  Ctx* c = s->c;
  const int nx = c->grid.nx, ny = c->grid.ny, nz = c->grid.nz;
  const int nxm = c->ax[0].nm, nym = c->ax[1].nm;
  T** p = reinterpret_cast<T**>(s->P);
  T *pp1 = p[0], *pgy1 = p[1], *pgz1 = p[2], *upi2 = p[3], *duy = p[4], *pp3 = p[5], *po3 = p[6];
  const int d1[3] = {nx, ny, nz};
  if (std::is_same<T, float>::value && c->st.istret == 0 && stag_fast_ok(c, 0, d1) && stag_fast_ok(c, 1, d1) &&
      stag_fast_ok(c, 2, d1)) {
    // binary32 periodic: circulant-form kernels, the y and z sums fused into
    // the solves (6 launches instead of 10)
    OpPlan *xd, *xi, *yd, *yi, *zd, *zi;
    RC(get_plan(c, 0, K_DVP, 0, default_coefset(K_DVP, 0), &xd));
    RC(get_plan(c, 0, K_IVP, 1, default_coefset(K_IVP, 1), &xi));
    RC(get_plan(c, 1, K_DVP, 0, default_coefset(K_DVP, 0), &yd));
    RC(get_plan(c, 1, K_IVP, 1, default_coefset(K_IVP, 1), &yi));
    RC(get_plan(c, 2, K_DVP, 0, default_coefset(K_DVP, 0), &zd));
    RC(get_plan(c, 2, K_IVP, 1, default_coefset(K_IVP, 1), &zi));
    float *f1 = (float*)pp1, *fy = (float*)pgy1, *fz = (float*)pgz1, *fu = (float*)upi2, *fd = (float*)duy;
    RC(stag_one(c, xd, f1, (const float*)ux, d1, st));
    RC(stag_one(c, xi, fy, (const float*)uy, d1, st));
    RC(stag_one(c, xi, fz, (const float*)uz, d1, st));
    RC(stag_sum(c, yd, fy, yi, f1, fd, false, d1, st));  // duy = deryvp(pgy1) + interyvp(pp1)
    RC(op<T>(s, 1, K_IVP, 1, upi2, pgz1, d1, st));       // upi2 = interyvp(pgz1)
    RC(stag_sum(c, zi, fd, zd, fu, pout, out64, d1, st)); // pp3 = interzvp(duy) + derzvp(upi2)
    s->launches += 5;
    return X3D_OK;
  }
  RC(op<T>(s, 0, K_DVP, 0, pp1, ux, d1, st));
  RC(op<T>(s, 0, K_IVP, 1, pgy1, uy, d1, st));
  RC(op<T>(s, 0, K_IVP, 1, pgz1, uz, d1, st));
  const int d2[3] = {nxm, ny, nz};
  RC(op<T>(s, 1, K_IVP, 1, upi2, pp1, d2, st));
  RC(op<T>(s, 1, K_DVP, 0, duy, pgy1, d2, st, nullptr, ymetric<T>(s, 3)));
  const long long n2 = (long long)nxm * c->ax[1].nm * nz;
  k_add<T><<<pw_blocks(c, n2), 256, 0, st>>>(duy, duy, upi2, n2);
  s->launches++;
  RC(op<T>(s, 1, K_IVP, 1, upi2, pgz1, d2, st));
  const int d3[3] = {nxm, nym, nz};
  RC(op<T>(s, 2, K_IVP, 1, pp3, duy, d3, st));
  RC(op<T>(s, 2, K_DVP, 0, po3, upi2, d3, st));
  if (out64) k_add_to64<T><<<pw_blocks(c, s->Np), 256, 0, st>>>((double*)pout, pp3, po3, s->Np);
  else k_add<T><<<pw_blocks(c, s->Np), 256, 0, st>>>((T*)pout, pp3, po3, s->Np);
  s->launches++;
  return cuda_status(cudaGetLastError());
}

// gradp of src/navier.f90:386-432 (the wall-gradient storage of the channel
// case is done by the caller).
// cor_h / cor_l (binary32 periodic path only): the double-float velocity
// components are corrected by the last (x-line) kernel of each gradient
// component instead of writing px, py, pz (*corrected tells which happened).
template <typename T>
static int gradp(SolverImpl* s, const T* pp3, T* px, T* py, T* pz, cudaStream_t st, float* const* cor_h = nullptr,
                 float* const* cor_l = nullptr, bool* corrected = nullptr) {
  if (corrected) *corrected = false;
  Ctx* c = s->c;
  const int ny = c->grid.ny, nz = c->grid.nz;
  const int nxm = c->ax[0].nm, nym = c->ax[1].nm, nzm = c->ax[2].nm;
  T** p = reinterpret_cast<T**>(s->P);
  T *ppi3 = p[0], *pgz3 = p[1], *ppi2 = p[2], *pgy2 = p[3], *pgzi2 = p[4];
  const int d3[3] = {nxm, nym, nzm};
  if (std::is_same<T, float>::value && c->st.istret == 0 && stag_fast_ok(c, 0, d3) && stag_fast_ok(c, 1, d3) &&
      stag_fast_ok(c, 2, d3)) {
    // binary32 periodic: circulant-form kernels, the z and y pairs on one
    // input fused (6 launches instead of 8)
    OpPlan *xd, *xi, *yd, *yi, *zd, *zi;
    RC(get_plan(c, 0, K_DPV, 1, default_coefset(K_DPV, 1), &xd));
    RC(get_plan(c, 0, K_IPV, 1, default_coefset(K_IPV, 1), &xi));
    RC(get_plan(c, 1, K_DPV, 1, default_coefset(K_DPV, 1), &yd));
    RC(get_plan(c, 1, K_IPV, 1, default_coefset(K_IPV, 1), &yi));
    RC(get_plan(c, 2, K_DPV, 1, default_coefset(K_DPV, 1), &zd));
    RC(get_plan(c, 2, K_IPV, 1, default_coefset(K_IPV, 1), &zi));
    float *f3 = (float*)ppi3, *f2 = (float*)ppi2, *fy = (float*)pgy2, *fzi = (float*)pgzi2;
    RC(stag_dual(c, zi, f3, zd, (float*)pgz3, (const float*)pp3, d3, st));  // ppi3, pgz3
    RC(stag_dual(c, yi, f2, yd, fy, f3, d3, st));                 // ppi2, pgy2
    RC(op<T>(s, 1, K_IPV, 1, pgzi2, pgz3, d3, st));                // pgzi2
    if (cor_h && cor_l) {
      RC(stag_one(c, xd, nullptr, f2, d3, st, cor_h[0], cor_l[0]));
      RC(stag_one(c, xi, nullptr, fy, d3, st, cor_h[1], cor_l[1]));
      RC(stag_one(c, xi, nullptr, fzi, d3, st, cor_h[2], cor_l[2]));
      if (corrected) *corrected = true;
    } else {
      RC(stag_one(c, xd, (float*)px, f2, d3, st));
      RC(stag_one(c, xi, (float*)py, fy, d3, st));
      RC(stag_one(c, xi, (float*)pz, fzi, d3, st));
    }
    s->launches += 5;
    return X3D_OK;
  }
  RC(op<T>(s, 2, K_IPV, 1, ppi3, pp3, d3, st));
  RC(op<T>(s, 2, K_DPV, 1, pgz3, pp3, d3, st));
  const int d2[3] = {nxm, nym, nz};
  RC(op<T>(s, 1, K_IPV, 1, ppi2, ppi3, d2, st));
  RC(op<T>(s, 1, K_DPV, 1, pgy2, ppi3, d2, st, nullptr, ymetric<T>(s, 0)));
  RC(op<T>(s, 1, K_IPV, 1, pgzi2, pgz3, d2, st));
  const int d1[3] = {nxm, ny, nz};
  RC(op<T>(s, 0, K_DPV, 1, px, ppi2, d1, st));
  RC(op<T>(s, 0, K_IPV, 1, py, pgy2, d1, st));
  RC(op<T>(s, 0, K_IPV, 1, pz, pgzi2, d1, st));
  return X3D_OK;
}

// ---- explicit LES host side ------------------------------------------------
// Work-field slots of the LES (FP64, N each)
enum {
  LW_P = 0,      // 6: products, filtered, then the Leonard stress L_ij
  LW_UF = 6,     // 3: filtered velocity
  LW_T = 9,      // 2: filter ping-pong
  LW_SF = 11,    // 6: strain of the filtered velocity, then b_ij
  LW_S = 17,     // 6: strain of the velocity
  LW_SRT = 23,   // 1: S:S
  LW_A = 24,     // 6: a_ij, then filtered
  LW_C = 30,     // 1: dynamic constant
  LW_NUT = 31,   // 1: eddy viscosity
  LW_G = 32,     // 3: SGS force
  LW_D = 35,     // 4: derivatives for the SGS force
  LW_COUNT = 39
};

// One dynsmag filter pass (alpha = 0 filter context).
static int les_fil(SolverImpl* s, int axis, int npaire, double* out, const double* in, cudaStream_t st) {
  Ctx* f = reinterpret_cast<Ctx*>(s->cf);
  OpPlan* p = nullptr;
  int rc = get_plan(f, axis, K_FIL, npaire, default_coefset(K_FIL, npaire), &p);
  if (rc != X3D_OK) return rc;
  const int dims[3] = {f->grid.nx, f->grid.ny, f->grid.nz};
  s->launches++;
  return launch_line_op<double>(f, p, out, in, dims, nullptr, st, nullptr);
}
static int les_fil3(SolverImpl* s, const double* u, int px, int py, int pz, double* out, cudaStream_t st) {
  double *a = s->lw[LW_T], *b = s->lw[LW_T + 1];
  RC(les_fil(s, 0, px, a, u, st));
  RC(les_fil(s, 1, py, b, a, st));
  return les_fil(s, 2, pz, out, b, st);
}

// Strain-rate tensor (sxx, syy, szz, sxy, sxz, syz) of smag
// (src/les_models.f90:190-263); tmp is scratch.
static int les_strain(SolverImpl* s, const double* ux, const double* uy, const double* uz, double* const* S,
                      double* tmp, cudaStream_t st) {
  const int dims[3] = {s->c->grid.nx, s->c->grid.ny, s->c->grid.nz};
  const double* ppy = ymetric<double>(s, 0);
  RC(op<double>(s, 0, K_DER1, 0, S[0], ux, dims, st));
  RC(op<double>(s, 1, K_DER1, 0, S[1], uy, dims, st, nullptr, ppy));
  RC(op<double>(s, 2, K_DER1, 0, S[2], uz, dims, st));
  Fuse<double> f = fz_comb<double>(0.5, tmp, 0.5, nullptr, 0.0, nullptr);  // 0.5 (t + tmp), exact halving
  RC(op<double>(s, 0, K_DER1, 1, tmp, uy, dims, st));                   // gyx
  RC(op<double>(s, 1, K_DER1, 1, S[3], ux, dims, st, &f, ppy));          // sxy = (gxy + gyx)/2
  RC(op<double>(s, 2, K_DER1, 1, tmp, ux, dims, st));                   // gxz
  RC(op<double>(s, 0, K_DER1, 1, S[4], uz, dims, st, &f));               // sxz = (gzx + gxz)/2
  RC(op<double>(s, 1, K_DER1, 1, tmp, uz, dims, st, nullptr, ppy));      // gzy
  RC(op<double>(s, 2, K_DER1, 1, S[5], uy, dims, st, &f));               // syz = (gyz + gzy)/2
  return X3D_OK;
}

// compute_SGS (src/les_models.f90:96-165, iconserv = 0): eddy viscosity into
// lw[LW_NUT] and the SGS force into lw[LW_G..LW_G+2].
static int les_compute(SolverImpl* s, const double* ux, const double* uy, const double* uz, cudaStream_t st) {
  Ctx* c = s->c;
  const long long N = s->N;
  const unsigned nb = pw_blocks(c, N);
  const int nx = c->grid.nx, ny = c->grid.ny, nz = c->grid.nz;
  double** w = s->lw;
  double* S[6] = {w[LW_S], w[LW_S + 1], w[LW_S + 2], w[LW_S + 3], w[LW_S + 4], w[LW_S + 5]};
  CSix cS = {{S[0], S[1], S[2], S[3], S[4], S[5]}};
  if (s->jles == 3) {
    // dynsmag (src/les_models.f90:333-903)
    double* P[6] = {w[LW_P], w[LW_P + 1], w[LW_P + 2], w[LW_P + 3], w[LW_P + 4], w[LW_P + 5]};
    k_les_prod<<<nb, 256, 0, st>>>(P[0], P[1], P[2], P[3], P[4], P[5], ux, uy, uz, N);
    s->launches++;
    double* uf[3] = {w[LW_UF], w[LW_UF + 1], w[LW_UF + 2]};
    RC(les_fil3(s, ux, 0, 1, 1, uf[0], st));
    RC(les_fil3(s, uy, 1, 0, 1, uf[1], st));
    RC(les_fil3(s, uz, 1, 1, 0, uf[2], st));
    const int pp[6][3] = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
    for (int q = 0; q < 6; ++q) RC(les_fil3(s, P[q], pp[q][0], pp[q][1], pp[q][2], P[q], st));
    k_les_leonard<<<nb, 256, 0, st>>>(Six{{P[0], P[1], P[2], P[3], P[4], P[5]}}, uf[0], uf[1], uf[2], N);
    s->launches++;
    double* SF[6] = {w[LW_SF], w[LW_SF + 1], w[LW_SF + 2], w[LW_SF + 3], w[LW_SF + 4], w[LW_SF + 5]};
    RC(les_strain(s, uf[0], uf[1], uf[2], SF, w[LW_T], st));
    RC(les_strain(s, ux, uy, uz, S, w[LW_T], st));
    Six bb = {{SF[0], SF[1], SF[2], SF[3], SF[4], SF[5]}};
    k_les_tensor<<<nb, 256, 0, st>>>(bb, CSix{{SF[0], SF[1], SF[2], SF[3], SF[4], SF[5]}}, s->del, 2.0, nx, ny, N);
    double* A[6] = {w[LW_A], w[LW_A + 1], w[LW_A + 2], w[LW_A + 3], w[LW_A + 4], w[LW_A + 5]};
    k_les_tensor<<<nb, 256, 0, st>>>(Six{{A[0], A[1], A[2], A[3], A[4], A[5]}}, cS, s->del, 1.0, nx, ny, N);
    k_les_srt<<<nb, 256, 0, st>>>(w[LW_SRT], cS, N);
    s->launches += 3;
    for (int q = 0; q < 6; ++q) RC(les_fil3(s, A[q], pp[q][0], pp[q][1], pp[q][2], A[q], st));
    k_les_smagc<<<nb, 256, 0, st>>>(w[LW_C], CSix{{P[0], P[1], P[2], P[3], P[4], P[5]}},
                                    CSix{{SF[0], SF[1], SF[2], SF[3], SF[4], SF[5]}},
                                    CSix{{A[0], A[1], A[2], A[3], A[4], A[5]}}, s->maxdsmagcst, N);
    s->launches++;
    RC(les_fil3(s, w[LW_C], 0, 0, 0, w[LW_C], st));
    k_les_nut_dyn<<<pw_blocks(c, (long long)nx * ny), 256, 0, st>>>(w[LW_NUT], w[LW_C], w[LW_SRT], s->del, nx, ny,
                                                                     nz);
    s->launches++;
  } else {
    // smag (src/les_models.f90:168-331)
    RC(les_strain(s, ux, uy, uz, S, w[LW_T], st));
    k_les_srt<<<nb, 256, 0, st>>>(w[LW_SRT], cS, N);
    k_les_nut_smag<<<nb, 256, 0, st>>>(w[LW_NUT], w[LW_SRT], s->del, s->smagcst, nx, ny, N);
    s->launches += 2;
  }
  // sgs_mom_nonconservative (src/les_models.f90:1091-1250)
  const int dims[3] = {nx, ny, nz};
  double *nut = w[LW_NUT], *gx = w[LW_G], *gy = w[LW_G + 1], *gz = w[LW_G + 2];
  double *ta = w[LW_D], *td = w[LW_D + 1], *te = w[LW_D + 2], *tf = w[LW_D + 3];
  const double* ppy = ymetric<double>(s, 0);
  RC(op<double>(s, 0, K_DER1, 1, ta, nut, dims, st));
  RC(op<double>(s, 0, K_DER2, 0, td, ux, dims, st));
  RC(op<double>(s, 0, K_DER2, 1, te, uy, dims, st));
  RC(op<double>(s, 0, K_DER2, 1, tf, uz, dims, st));
  k_les_sgs<<<nb, 256, 0, st>>>(gx, gy, gz, td, te, tf, nut, ta, S[0], S[3], S[4], 1, N);
  RC(op<double>(s, 1, K_DER1, 1, ta, nut, dims, st, nullptr, ppy));
  const double* us[3] = {ux, uy, uz};
  double* ts[3] = {td, te, tf};
  const int par[3] = {1, 0, 1};
  for (int q = 0; q < 3; ++q) {
    RC(op<double>(s, 1, K_DER2, par[q], ts[q], us[q], dims, st));
    if (ppy) {
      RC(op<double>(s, 1, K_DER1, par[q], w[LW_T], us[q], dims, st, nullptr, ppy));
      k_stretch_d2<<<nb, 256, 0, st>>>(ts[q], w[LW_T], ymetric<double>(s, 1), ymetric<double>(s, 2), nx, ny, N);
      s->launches++;
    }
  }
  k_les_sgs<<<nb, 256, 0, st>>>(gx, gy, gz, td, te, tf, nut, ta, S[3], S[1], S[5], 0, N);
  RC(op<double>(s, 2, K_DER1, 1, ta, nut, dims, st));
  RC(op<double>(s, 2, K_DER2, 1, td, ux, dims, st));
  RC(op<double>(s, 2, K_DER2, 1, te, uy, dims, st));
  RC(op<double>(s, 2, K_DER2, 0, tf, uz, dims, st));
  k_les_sgs<<<nb, 256, 0, st>>>(gx, gy, gz, td, te, tf, nut, ta, S[4], S[5], S[2], 0, N);
  s->launches += 3;
  return cuda_status(cudaGetLastError());
}

// Learned closure: tau_ij from the MLP on the 9 velocity gradients, force
// -d_j tau_ij into lw[LW_G..LW_G+2].
static int les_mlp_force(SolverImpl* s, const double* ux, const double* uy, const double* uz, cudaStream_t st) {
  Ctx* c = s->c;
  const long long N = s->N;
  const int dims[3] = {c->grid.nx, c->grid.ny, c->grid.nz};
  double** w = s->lw;
  const double* ppy = ymetric<double>(s, 0);
  const double* U[3] = {ux, uy, uz};
  double* g[9];
  for (int q = 0; q < 9; ++q) g[q] = w[LW_P + q];  // slots LW_P .. LW_P+8
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const int np = (i == j) ? 0 : 1;
      RC(op<double>(s, j, K_DER1, np, g[3 * i + j], U[i], dims, st, nullptr, j == 1 ? ppy : nullptr));
    }
  double* tau[6];
  for (int q = 0; q < 6; ++q) tau[q] = w[LW_S + q];
  const double delta = std::cbrt(c->ax[0].d * c->ax[1].d * c->ax[2].d);
  RC(mlp_les_tau(s->mlp, g, delta, tau, N, c->num_sms, st));
  s->launches++;
  // f_i = -(d_x tau_ix + d_y tau_iy + d_z tau_iz)
  const int ti[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
  const int pt[6][3] = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  for (int i = 0; i < 3; ++i) {
    double* G = w[LW_G + i];
    for (int j = 0; j < 3; ++j) {
      const int q = ti[i][j];
      // G = -d_j tau_ij (+ G)
      Fuse<double> f = fz_comb<double>(-1.0, j == 0 ? nullptr : G, 1.0, nullptr, 0.0, nullptr);
      RC(op<double>(s, j, K_DER1, pt[q][j], G, tau[q], dims, st, &f, j == 1 ? ppy : nullptr));
    }
  }
  return cuda_status(cudaGetLastError());
}

// ppy as channel_cfr divides by it: the stretching metric, or on a uniform
// mesh the default 1 with 2 at the walls (src/variables.f90:1294-1305).
static const double* ymetric_cfr(SolverImpl* s) {
  const double* d = nullptr;
  if (stretch_device(s->c, &d) != X3D_OK) return nullptr;
  return d;
}

template <typename T>
static int substep(SolverImpl* s, int itr, cudaStream_t st) {
  Ctx* c = s->c;
  const long long N = s->N;
  const unsigned nb = pw_blocks(c, N);
  const bool mixed = std::is_same<T, float>::value;
  // operator inputs: the FP64 state, or the hi part of the double-float state
  const T* u[3];
  for (int q = 0; q < 3; ++q) u[q] = mixed ? (const T*)s->uh[q] : (const T*)(q == 0 ? s->ux : q == 1 ? s->uy : s->uz);
  T* H[3] = {(T*)s->H[0][0], (T*)s->H[1][0], (T*)s->H[2][0]};
  const int it = s->itime + 1;  // 1-based step index
  if (s->cfr) {
    // boundary_conditions -> channel_cfr on ux, before the right-hand side
    const int np = 2 * c->num_sms;
    k_cfr_partial<<<np, 256, 0, st>>>(s->ux, ymetric_cfr(s), c->grid.nx, c->grid.ny, N, s->part);
    const double coeff = c->ax[1].d / (c->grid.yly * (double)(c->grid.nx * c->grid.nz));
    k_cfr_finish<<<1, 256, 0, st>>>(s->part, np, coeff, s->cfr_target, s->ub_dev + 2 * (itr - 1));
    k_sub_dev<<<nb, 256, 0, st>>>(s->ux, s->ub_dev + 2 * (itr - 1) + 1, N);
    s->launches += 3;
  }
  RC(momentum_rhs<T>(s, u, H, st));
  if (s->jles != 0) {
    // src/transeq.f90:475-480: the SGS force joins the right-hand side
    if (s->jles == 10) {
      RC(les_mlp_force(s, s->ux, s->uy, s->uz, st));
    } else {
      RC(les_compute(s, s->ux, s->uy, s->uz, st));
    }
    k_add3<<<nb, 256, 0, st>>>((double*)H[0], (double*)H[1], (double*)H[2], s->lw[LW_G], s->lw[LW_G + 1],
                               s->lw[LW_G + 2], N);
    s->launches++;
  }
  if (s->walls && s->wrotation != 0.0 && it < s->spinup_time) {
    k_rotation<<<nb, 256, 0, st>>>((double*)H[0], (double*)H[1], s->ux, s->uy, s->wrotation, N);
    s->launches++;
  }
  // intt (src/time_integrators.f90:18-187)
  const double dt = s->o.dt;
  double c1 = 0, c2 = 0, c3 = 0;
  int nh = 1;
  if (s->o.itimescheme == 3) {
    if (it == 1) { c1 = dt; nh = 1; }
    else if (it == 2) { c1 = 1.5 * dt; c2 = -0.5 * dt; nh = 2; }
    else { c1 = s->adt[0]; c2 = s->bdt[0]; c3 = s->cdt[0]; nh = 3; }
  } else {
    if (itr == 1) { c1 = s->gdt[0]; nh = 1; }
    else { c1 = s->adt[itr - 1]; c2 = s->bdt[itr - 1]; nh = 2; }
  }
  if (mixed) {
    Intt3 a;
    for (int q = 0; q < 3; ++q) {
      a.uh[q] = s->uh[q];
      a.ul[q] = s->ul[q];
      for (int k = 0; k < 3; ++k) a.h[q][k] = (const float*)s->H[q][k];
    }
    if (N % 4 == 0) k_intt_df4<<<nb, 256, 0, st>>>(a, (float)c1, (float)c2, (float)c3, nh, N / 4);
    else k_intt_df<<<nb, 256, 0, st>>>(a, (float)c1, (float)c2, (float)c3, nh, N);
    s->launches++;
  } else {
    double* U[3] = {s->ux, s->uy, s->uz};
    for (int q = 0; q < 3; ++q) {
      k_intt64<<<nb, 256, 0, st>>>(U[q], (const double*)s->H[q][0], (const double*)s->H[q][1],
                                   (const double*)s->H[q][2], c1, c2, c3, nh, N);
      s->launches++;
    }
  }
  // history rotation: dvar(3)=dvar(2); dvar(2)=dvar(1)
  for (int q = 0; q < 3; ++q) {
    if (s->ntime == 3) {
      void* t = s->H[q][2];
      s->H[q][2] = s->H[q][1];
      s->H[q][1] = s->H[q][0];
      s->H[q][0] = t;
    } else {
      void* t = s->H[q][1];
      s->H[q][1] = s->H[q][0];
      s->H[q][0] = t;
    }
  }
  RC(cuda_status(cudaGetLastError()));
  const double g = s->gdt[s->o.itimescheme == 3 ? 0 : itr - 1];
  if (s->walls) {
    k_walls<<<pw_blocks(c, (long long)c->grid.nx * c->grid.nz), 256, 0, st>>>(
        s->ux, s->uy, s->uz, s->wall_dp, g, c->grid.nx, c->grid.ny, c->grid.nz);
    s->launches++;
  }
  // projection: divergence, Poisson, gradient, correction
  T** w = reinterpret_cast<T**>(s->W);
  const T* pin = (const T*)s->pp64;
  if (mixed) {
    // binary32 divergence -> FP64-class Poisson solve in double-float
    // arithmetic on the FP32 pipes -> binary32 pressure (rounded once)
    RC(divergence<T>(s, u[0], u[1], u[2], s->p32, false, st));
    RC(poisson_periodic_f32io(c, s->p32, st));
    pin = (const T*)s->p32;
  } else {
    RC(divergence<T>(s, u[0], u[1], u[2], s->pp64, true, st));
    if (s->walls) {
      RC(poisson_010(c, s->pp64, st));
    } else if (s->slip) {
      RC(poisson_11x(c, s->pp64, st));
    } else {
      RC(poisson_periodic(c, s->pp64, 0, st));
    }
  }
  s->launches += 5;
  bool corrected = false;
  if (mixed && !s->walls)
    RC(gradp<T>(s, pin, w[0], w[1], w[2], st, s->uh, s->ul, &corrected));
  else
    RC(gradp<T>(s, pin, w[0], w[1], w[2], st));
  if (s->walls) {
    k_wallgrad<<<pw_blocks(c, (long long)c->grid.nx * c->grid.nz), 256, 0, st>>>(
        s->wall_dp, (const double*)w[0], (const double*)w[2], g, c->grid.nx, c->grid.ny, c->grid.nz);
    s->launches++;
  }
  if (corrected) return cuda_status(cudaGetLastError());  // cor_vel done by the gradient kernels
  if (mixed) {
    Cor3 a;
    for (int q = 0; q < 3; ++q) {
      a.uh[q] = s->uh[q];
      a.ul[q] = s->ul[q];
      a.p[q] = (const float*)w[q];
    }
    if (N % 4 == 0) k_corvel_df4<<<nb, 256, 0, st>>>(a, N / 4);
    else k_corvel_df<<<nb, 256, 0, st>>>(a, N);
  } else {
    k_corvel<T><<<nb, 256, 0, st>>>(s->ux, s->uy, s->uz, w[0], w[1], w[2], N);
  }
  s->launches++;
  return cuda_status(cudaGetLastError());
}

static int solver_alloc(SolverImpl* s) {
  Ctx* c = s->c;
  const long long N = s->N;
  const bool mixed = s->mixed();
  const size_t es = mixed ? sizeof(float) : sizeof(double);
  s->ux = s->alloc<double>(N);
  s->uy = s->alloc<double>(N);
  s->uz = s->alloc<double>(N);
  if (!s->ux || !s->uy || !s->uz) return X3D_ERR_NOMEM;
  if (mixed) {
    for (int q = 0; q < 3; ++q) {
      s->uh[q] = s->alloc<float>(N);
      s->ul[q] = s->alloc<float>(N);
      if (!s->uh[q] || !s->ul[q]) return X3D_ERR_NOMEM;
    }
  }
  for (int q = 0; q < 3; ++q)
    for (int k = 0; k < s->ntime; ++k) {
      s->H[q][k] = s->alloc<unsigned char>(N * (long long)es);
      if (!s->H[q][k]) return X3D_ERR_NOMEM;
      cudaMemset(s->H[q][k], 0, (size_t)N * es);
    }
  const int nw = (c->st.istret != 0) ? 7 : 5;
  for (int k = 0; k < nw; ++k) {
    s->W[k] = s->alloc<unsigned char>(N * (long long)es);
    if (!s->W[k]) return X3D_ERR_NOMEM;
  }
  if (s->walls) {
    const long long nwall = 4LL * c->grid.nx * c->grid.nz;
    s->wall_dp = s->alloc<double>(nwall);
    s->ub_dev = s->alloc<double>(6);
    if (!s->wall_dp || !s->ub_dev) return X3D_ERR_NOMEM;
    cudaMemset(s->wall_dp, 0, (size_t)nwall * sizeof(double));
    cudaMemset(s->ub_dev, 0, 6 * sizeof(double));
  }
  for (int k = 0; k < 7; ++k) {
    s->P[k] = s->alloc<unsigned char>(N * (long long)es);
    if (!s->P[k]) return X3D_ERR_NOMEM;
  }
  if (mixed) {
    s->p32 = s->alloc<float>(N);
    if (!s->p32) return X3D_ERR_NOMEM;
  } else {
    s->pp64 = s->alloc<double>(N);
    if (!s->pp64) return X3D_ERR_NOMEM;
  }
  s->part = s->alloc<double>(4LL * 4096);
  if (!s->part) return X3D_ERR_NOMEM;
  if (cudaMallocHost(&s->hpart, 4 * 4096 * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
  return cuda_status(cudaGetLastError());
}

}  // namespace x3d

using namespace x3d;

extern "C" {

int x3d_solver_create(x3d_ctx* ctx_, const x3d_solver_opts* o, x3d_solver** out) {
  if (!ctx_ || !o || !out) return X3D_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(ctx_);
  const bool periodic = c->ax[0].periodic && c->ax[1].periodic && c->ax[2].periodic;
  // channel geometry: x, z periodic, no-slip walls at both y ends
  const bool walls = c->ax[0].periodic && c->ax[2].periodic && !c->ax[1].periodic && c->ax[1].ncl1 == 2 &&
                     c->ax[1].ncln == 2;
  // free-slip box (the reference's TGV test case): x and y free-slip, z free-slip or periodic
  const bool slip = is_11x(c);
  if (!periodic && !walls && !slip) return X3D_ERR_BC;
  if (o->itimescheme != 3 && o->itimescheme != 5) return X3D_ERR_UNSUPPORTED;
  if (o->precision != X3D_PREC_FP64 && o->precision != X3D_PREC_MIXED) return X3D_ERR_DTYPE;
  if ((walls || slip) && o->precision != X3D_PREC_FP64) return X3D_ERR_DTYPE;
  if (slip && c->st.istret != 0) return X3D_ERR_UNSUPPORTED;
  if (walls && c->st.istret == 3) return X3D_ERR_UNSUPPORTED;
  x3d_solver* s = new x3d_solver();
  SolverImpl* si = &s->impl;
  si->c = c;
  si->o = *o;
  si->walls = walls;
  si->slip = slip;
  si->N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
  si->Np = (long long)c->ax[0].nm * c->ax[1].nm * c->ax[2].nm;
  const double dt = o->dt;
  if (o->itimescheme == 3) {  // src/variables.f90:1366-1377
    si->ntime = 3; si->nsub = 1;
    si->adt[0] = (23.0 / 12.0) * dt; si->bdt[0] = -(16.0 / 12.0) * dt; si->cdt[0] = (5.0 / 12.0) * dt;
    si->gdt[0] = si->adt[0] + si->bdt[0] + si->cdt[0];
  } else {  // RK3, src/variables.f90:1389-1400
    si->ntime = 2; si->nsub = 3;
    si->adt[0] = (8.0 / 15.0) * dt; si->bdt[0] = 0.0; si->gdt[0] = si->adt[0];
    si->adt[1] = (5.0 / 12.0) * dt; si->bdt[1] = (-17.0 / 60.0) * dt; si->gdt[1] = si->adt[1] + si->bdt[1];
    si->adt[2] = (3.0 / 4.0) * dt; si->bdt[2] = (-5.0 / 12.0) * dt; si->gdt[2] = si->adt[2] + si->bdt[2];
  }
  int rc = solver_alloc(si);
  if (rc != X3D_OK) {
    delete s;
    return rc;
  }
  *out = s;
  return X3D_OK;
}

int x3d_solver_destroy(x3d_solver* s) {
  delete s;
  return X3D_OK;
}

int x3d_solver_set_channel(x3d_solver* s, double target_ub, double wrotation, int spinup_time) {
  if (!s) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  if (!si->walls) return X3D_ERR_BC;
  si->cfr = true;
  si->cfr_target = target_ub;
  si->wrotation = wrotation;
  si->spinup_time = spinup_time;
  return X3D_OK;
}

int x3d_solver_set_les(x3d_solver* s, int jles, double smagcst, double maxdsmagcst) {
  if (!s) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  if (jles != 0 && jles != 1 && jles != 3) return X3D_ERR_UNSUPPORTED;
  if (si->mixed()) return X3D_ERR_DTYPE;
  Ctx* c = si->c;
  if (jles != 0 && !si->lw[0]) {
    // filter width del(j) of init_explicit_les (src/les_models.f90:27-30)
    const int ny = c->grid.ny;
    std::vector<double> del(ny);
    for (int j = 0; j < ny - 1; ++j)
      del[j] = std::pow(c->ax[0].d * (c->st.yp[j + 1] - c->st.yp[j]) * c->ax[2].d, 1.0 / 3.0);
    del[ny - 1] = del[ny - 2];
    si->del = si->alloc<double>(ny);
    if (!si->del) return X3D_ERR_NOMEM;
    int rc = cuda_status(cudaMemcpy(si->del, del.data(), ny * sizeof(double), cudaMemcpyHostToDevice));
    if (rc != X3D_OK) return rc;
    // dynsmag filters with alpha = 0 (filter(zero), src/les_models.f90:393)
    x3d_numopts o = c->opts;
    o.filter_alpha = 0.0;
    rc = x3d_ctx_create(&c->grid, &o, &si->cf);
    if (rc != X3D_OK) return rc;
    for (int k = 0; k < LW_COUNT; ++k) {
      si->lw[k] = si->alloc<double>(si->N);
      if (!si->lw[k]) return X3D_ERR_NOMEM;
    }
  }
  si->jles = jles;
  si->smagcst = smagcst;
  si->maxdsmagcst = maxdsmagcst;
  return X3D_OK;
}

int x3d_solver_set_les_mlp(x3d_solver* s, x3d_mlp* m) {
  if (!s) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  if (!m) {
    si->mlp = nullptr;
    if (si->jles == 10) si->jles = 0;
    return X3D_OK;
  }
  int rc = x3d_solver_set_les(s, 1, si->smagcst, si->maxdsmagcst);  // work fields and filter width
  if (rc != X3D_OK) return rc;
  si->mlp = reinterpret_cast<Mlp*>(m);
  si->jles = 10;
  return X3D_OK;
}

int x3d_solver_les_fields(x3d_solver* s, double* nut, double* sgsx, double* sgsy, double* sgsz, void* stream) {
  if (!s || !nut || !sgsx || !sgsy || !sgsz) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  if (si->jles == 0) return X3D_ERR_STATE;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = X3D_OK;
  if (si->jles == 10) {
    rc = les_mlp_force(si, si->ux, si->uy, si->uz, st);
    if (rc == X3D_OK) rc = cuda_status(cudaMemsetAsync(si->lw[LW_NUT], 0, (size_t)si->N * sizeof(double), st));
  } else {
    rc = les_compute(si, si->ux, si->uy, si->uz, st);
  }
  if (rc != X3D_OK) return rc;
  const size_t b = (size_t)si->N * sizeof(double);
  double* dst[4] = {nut, sgsx, sgsy, sgsz};
  const double* src[4] = {si->lw[LW_NUT], si->lw[LW_G], si->lw[LW_G + 1], si->lw[LW_G + 2]};
  for (int q = 0; q < 4; ++q) {
    rc = cuda_status(cudaMemcpyAsync(dst[q], src[q], b, cudaMemcpyDeviceToDevice, st));
    if (rc != X3D_OK) return rc;
  }
  return X3D_OK;
}

int x3d_solver_bulk_velocity(x3d_solver* s, double* out, int capacity) {
  if (!s || !out) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  if (!si->cfr) return X3D_ERR_STATE;
  if (capacity < si->nsub) return X3D_ERR_ARG;
  double h[6];
  int rc = cuda_status(cudaMemcpy(h, si->ub_dev, sizeof(h), cudaMemcpyDeviceToHost));
  if (rc != X3D_OK) return rc;
  for (int k = 0; k < si->nsub; ++k) out[k] = h[2 * k];
  return si->nsub;
}

// After the FP64 staging arrays change: derive the double-float state.
static int sync_copies(SolverImpl* s) {
  if (!s->mixed()) return X3D_OK;
  Ctx* c = s->c;
  const unsigned nb = pw_blocks(c, s->N);
  const double* U[3] = {s->ux, s->uy, s->uz};
  for (int q = 0; q < 3; ++q) k_split<<<nb, 256>>>(s->uh[q], s->ul[q], U[q], s->N);
  return cuda_status(cudaDeviceSynchronize());
}

// Before reading the FP64 staging arrays: rebuild them from the double-float state.
static int stage64(SolverImpl* s, cudaStream_t st) {
  if (!s->mixed()) return X3D_OK;
  Ctx* c = s->c;
  const unsigned nb = pw_blocks(c, s->N);
  double* U[3] = {s->ux, s->uy, s->uz};
  for (int q = 0; q < 3; ++q) k_combine<<<nb, 256, 0, st>>>(U[q], s->uh[q], s->ul[q], s->N);
  return cuda_status(cudaGetLastError());
}

// Device-accessible address of a page-locked host buffer, or null.
static const void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

__global__ void k_copy64(double* d, const double* s, long long n) {
  GRID_STRIDE(i, n) d[i] = s[i];
}

// Host <-> device kernels of the asynchronous transfers: 16-byte accesses,
// four in flight per thread, two blocks per SM, so that the kernels of
// different components run side by side (one reading host memory while
// another writes it) instead of each filling the GPU in turn.
__global__ void __launch_bounds__(256) k_xin(float* uh, float* ul, double* u, const double* h, long long n2) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n2; i0 += 4 * stride) {
    double2 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const long long i = i0 + k * stride;
      if (i < n2) v[k] = reinterpret_cast<const double2*>(h)[i];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const long long i = i0 + k * stride;
      if (i >= n2) continue;
      if (u) {
        reinterpret_cast<double2*>(u)[i] = v[k];
      } else {
        const float hx = (float)v[k].x, hy = (float)v[k].y;
        reinterpret_cast<float2*>(uh)[i] = make_float2(hx, hy);
        reinterpret_cast<float2*>(ul)[i] = make_float2((float)(v[k].x - (double)hx), (float)(v[k].y - (double)hy));
      }
    }
  }
}
__global__ void __launch_bounds__(256) k_xout(double* h, const float* uh, const float* ul, const double* u,
                                              long long n2) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n2; i0 += 4 * stride) {
    double2 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const long long i = i0 + k * stride;
      if (i >= n2) continue;
      if (u) {
        v[k] = reinterpret_cast<const double2*>(u)[i];
      } else {
        const float2 a = reinterpret_cast<const float2*>(uh)[i], b = reinterpret_cast<const float2*>(ul)[i];
        v[k] = make_double2((double)a.x + (double)b.x, (double)a.y + (double)b.y);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const long long i = i0 + k * stride;
      if (i < n2) reinterpret_cast<double2*>(h)[i] = v[k];
    }
  }
}

static int xfer_setup(SolverImpl* si) {
  if (si->xfer_init) return X3D_OK;
  for (int q = 0; q < 3; ++q) {
    if (cudaStreamCreateWithFlags(&si->xs[q], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&si->ev_set[q], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&si->ev_get[q], cudaEventDisableTiming) != cudaSuccess)
      return X3D_ERR_CUDA;
  }
  if (cudaEventCreateWithFlags(&si->ev_step, cudaEventDisableTiming) != cudaSuccess) return X3D_ERR_CUDA;
  si->xfer_init = true;
  return X3D_OK;
}

// Work on the transfer streams must be finished before a synchronous call
// touches the state or the host buffers.
static void xfer_drain(SolverImpl* si) {
  if (si->xfer_init)
    for (int q = 0; q < 3; ++q) cudaStreamSynchronize(si->xs[q]);
}

int x3d_solver_set_velocity_async(x3d_solver* s, const double* ux, const double* uy, const double* uz,
                                  void* stream) {
  if (!s || !ux || !uy || !uz) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  const void* m[3] = {mapped_host(ux), mapped_host(uy), mapped_host(uz)};
  if (!m[0] || !m[1] || !m[2]) return X3D_ERR_ARG;  // page-locked host memory only
  int rc = xfer_setup(si);
  if (rc != X3D_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // write-ins run in order on the second transfer stream, after the work
  // already queued on the caller's stream (the previous step) and each after
  // its own component's previous read-out (same host buffer, same state):
  // write-in of u overlaps the read-out of v, and so on
  cudaEventRecord(si->ev_step, st);
  cudaStream_t xw = si->xs[1];
  cudaStreamWaitEvent(xw, si->ev_step, 0);
  const bool vec = (si->N % 2 == 0);
  const unsigned nb = vec ? (unsigned)(2 * si->c->num_sms) : pw_blocks(si->c, si->N);
  double* U[3] = {si->ux, si->uy, si->uz};
  for (int q = 0; q < 3; ++q) {
    cudaStreamWaitEvent(xw, si->ev_get[q], 0);
    if (vec)
      k_xin<<<nb, 256, 0, xw>>>(si->mixed() ? si->uh[q] : nullptr, si->mixed() ? si->ul[q] : nullptr,
                                si->mixed() ? nullptr : U[q], (const double*)m[q], si->N / 2);
    else if (si->mixed())
      k_split<<<nb, 256, 0, xw>>>(si->uh[q], si->ul[q], (const double*)m[q], si->N);
    else
      k_copy64<<<nb, 256, 0, xw>>>(U[q], (const double*)m[q], si->N);
    cudaEventRecord(si->ev_set[q], xw);
  }
  cudaStreamWaitEvent(st, si->ev_set[2], 0);
  return cuda_status(cudaGetLastError());
}

int x3d_solver_get_velocity_async(x3d_solver* s, double* ux, double* uy, double* uz, void* stream) {
  if (!s || !ux || !uy || !uz) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  void* m[3] = {(void*)mapped_host(ux), (void*)mapped_host(uy), (void*)mapped_host(uz)};
  if (!m[0] || !m[1] || !m[2]) return X3D_ERR_ARG;
  int rc = xfer_setup(si);
  if (rc != X3D_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // read-outs in order u, v, w on the first transfer stream
  cudaEventRecord(si->ev_step, st);
  cudaStream_t xr = si->xs[0];
  cudaStreamWaitEvent(xr, si->ev_step, 0);
  const bool vec = (si->N % 2 == 0);
  const unsigned nb = vec ? (unsigned)(2 * si->c->num_sms) : pw_blocks(si->c, si->N);
  double* U[3] = {si->ux, si->uy, si->uz};
  for (int q = 0; q < 3; ++q) {
    if (vec)
      k_xout<<<nb, 256, 0, xr>>>((double*)m[q], si->mixed() ? si->uh[q] : nullptr,
                                 si->mixed() ? si->ul[q] : nullptr, si->mixed() ? nullptr : U[q], si->N / 2);
    else if (si->mixed())
      k_combine<<<nb, 256, 0, xr>>>((double*)m[q], si->uh[q], si->ul[q], si->N);
    else
      k_copy64<<<nb, 256, 0, xr>>>((double*)m[q], U[q], si->N);
    cudaEventRecord(si->ev_get[q], xr);
  }
  return cuda_status(cudaGetLastError());
}

int x3d_solver_sync(x3d_solver* s) {
  if (!s) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  xfer_drain(si);
  return cuda_status(cudaDeviceSynchronize());
}

int x3d_solver_set_velocity(x3d_solver* s, const double* ux, const double* uy, const double* uz, int on_device) {
  if (!s || !ux || !uy || !uz) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  xfer_drain(si);
  // Page-locked host buffers are read by the kernels directly (over the
  // host-device link), without a staging copy.
  if (!on_device) {
    const void* m[3] = {mapped_host(ux), mapped_host(uy), mapped_host(uz)};
    if (m[0] && m[1] && m[2]) {
      const unsigned nb = pw_blocks(si->c, si->N);
      double* U[3] = {si->ux, si->uy, si->uz};
      for (int q = 0; q < 3; ++q) {
        if (si->mixed()) k_split<<<nb, 256>>>(si->uh[q], si->ul[q], (const double*)m[q], si->N);
        else k_copy64<<<nb, 256>>>(U[q], (const double*)m[q], si->N);
      }
      si->itime = 0;
      return cuda_status(cudaDeviceSynchronize());
    }
  }
  const size_t b = (size_t)si->N * sizeof(double);
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (cudaMemcpy(si->ux, ux, b, k) != cudaSuccess || cudaMemcpy(si->uy, uy, b, k) != cudaSuccess ||
      cudaMemcpy(si->uz, uz, b, k) != cudaSuccess)
    return X3D_ERR_CUDA;
  si->itime = 0;
  return sync_copies(si);
}

int x3d_solver_get_velocity(x3d_solver* s, double* ux, double* uy, double* uz, int on_device) {
  if (!s || !ux || !uy || !uz) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  xfer_drain(si);
  if (!on_device) {
    void* m[3] = {(void*)mapped_host(ux), (void*)mapped_host(uy), (void*)mapped_host(uz)};
    if (m[0] && m[1] && m[2]) {
      const unsigned nb = pw_blocks(si->c, si->N);
      double* U[3] = {si->ux, si->uy, si->uz};
      for (int q = 0; q < 3; ++q) {
        if (si->mixed()) k_combine<<<nb, 256>>>((double*)m[q], si->uh[q], si->ul[q], si->N);
        else k_copy64<<<nb, 256>>>((double*)m[q], U[q], si->N);
      }
      return cuda_status(cudaDeviceSynchronize());
    }
  }
  int rc = stage64(si, nullptr);
  if (rc != X3D_OK) return rc;
  const size_t b = (size_t)si->N * sizeof(double);
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (cudaMemcpy(ux, si->ux, b, k) != cudaSuccess || cudaMemcpy(uy, si->uy, b, k) != cudaSuccess ||
      cudaMemcpy(uz, si->uz, b, k) != cudaSuccess)
    return X3D_ERR_CUDA;
  return X3D_OK;
}

// ---- restart state (src/tools.f90:205-514): history and pressure ---------
__global__ void k_f32_to_f64(double* o, const float* a, long long n) {
  GRID_STRIDE(i, n) o[i] = (double)a[i];
}

// which: 0..2 velocity, 3..5 previous right-hand side (dux-2, duy-2, duz-2),
// 6..8 the one before (dux-3, ...), 9 pressure (nxm, nym, nzm).
static int state_slot(SolverImpl* si, int which, void** ptr, long long* n, bool* f32) {
  *f32 = false;
  *n = si->N;
  if (which >= 0 && which <= 2) {
    *ptr = which == 0 ? si->ux : which == 1 ? si->uy : si->uz;
    return X3D_OK;
  }
  if (which >= 3 && which <= 8) {
    const int slot = which < 6 ? 1 : 2;
    if (slot >= si->ntime) return X3D_ERR_STATE;
    *ptr = si->H[(which - 3) % 3][slot];
    *f32 = si->mixed();
    return X3D_OK;
  }
  if (which == 9) {
    *ptr = si->mixed() ? (void*)si->p32 : (void*)si->pp64;
    *f32 = si->mixed();
    *n = si->Np;
    return X3D_OK;
  }
  return X3D_ERR_ARG;
}

int x3d_solver_get_field(x3d_solver* s, int which, double* out, int on_device) {
  if (!s || !out) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  xfer_drain(si);
  void* p = nullptr;
  long long n = 0;
  bool f32 = false;
  int rc = state_slot(si, which, &p, &n, &f32);
  if (rc != X3D_OK) return rc;
  if (which <= 2) {
    rc = stage64(si, nullptr);
    if (rc != X3D_OK) return rc;
  }
  const double* src = (const double*)p;
  if (f32) {
    // binary32 history of the mixed solver, widened through a temporary
    double* stage = nullptr;
    if (cudaMalloc(&stage, (size_t)n * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
    k_f32_to_f64<<<pw_blocks(si->c, n), 256>>>(stage, (const float*)p, n);
    rc = cuda_status(cudaMemcpy(out, stage, (size_t)n * sizeof(double),
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
    cudaFree(stage);
    return rc;
  }
  return cuda_status(cudaMemcpy(out, src, (size_t)n * sizeof(double),
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
}

int x3d_solver_set_field(x3d_solver* s, int which, const double* in, int on_device) {
  if (!s || !in) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  xfer_drain(si);
  void* p = nullptr;
  long long n = 0;
  bool f32 = false;
  int rc = state_slot(si, which, &p, &n, &f32);
  if (rc != X3D_OK) return rc;
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (f32) {
    double* stage = nullptr;
    if (cudaMalloc(&stage, (size_t)n * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
    rc = cuda_status(cudaMemcpy(stage, in, (size_t)n * sizeof(double), k));
    if (rc == X3D_OK) {
      k_to32<<<pw_blocks(si->c, n), 256>>>((float*)p, stage, n);
      rc = cuda_status(cudaDeviceSynchronize());
    }
    cudaFree(stage);
    return rc;
  }
  if (which <= 2 && si->mixed()) {
    rc = stage64(si, nullptr);  // the other components' staging must be current
    if (rc != X3D_OK) return rc;
  }
  rc = cuda_status(cudaMemcpy(p, in, (size_t)n * sizeof(double), k));
  if (rc == X3D_OK && which <= 2 && si->mixed()) rc = sync_copies(si);
  return rc;
}

int x3d_solver_get_itime(x3d_solver* s) {
  if (!s) return X3D_ERR_ARG;
  return s->impl.itime;
}

int x3d_solver_set_itime(x3d_solver* s, int itime) {
  if (!s || itime < 0) return X3D_ERR_ARG;
  s->impl.itime = itime;
  return X3D_OK;
}

int x3d_solver_init_tgv(x3d_solver* s) {
  if (!s) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  Ctx* c = si->c;
  k_tgv_init<<<pw_blocks(c, si->N), 256>>>(si->ux, si->uy, si->uz, c->grid.nx, c->grid.ny, c->grid.nz, c->ax[0].d,
                                           c->ax[1].d, c->ax[2].d);
  si->itime = 0;
  int rc = cuda_status(cudaGetLastError());
  if (rc != X3D_OK) return rc;
  return sync_copies(si);
}

int x3d_solver_step(x3d_solver* s, int nsteps, void* stream) {
  if (!s || nsteps < 0) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  cudaStream_t st = (cudaStream_t)stream;
  // asynchronous read-outs of the state still in flight finish first
  if (si->xfer_init)
    for (int q = 0; q < 3; ++q) cudaStreamWaitEvent(st, si->ev_get[q], 0);
  for (int n = 0; n < nsteps; ++n) {
    for (int itr = 1; itr <= si->nsub; ++itr) {
      const int rc = si->mixed() ? substep<float>(si, itr, st) : substep<double>(si, itr, st);
      if (rc != X3D_OK) return rc;
    }
    si->itime++;
  }
  return X3D_OK;
}

int x3d_solver_launches_per_step(x3d_solver* s) {
  if (!s) return X3D_ERR_ARG;
  return s->impl.launches / (s->impl.itime > 0 ? s->impl.itime : 1);
}

int x3d_solver_tgv_stats(x3d_solver* s, double* out, void* stream) {
  if (!s || !out) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  xfer_drain(si);
  Ctx* c = si->c;
  cudaStream_t st = (cudaStream_t)stream;
  const int dims[3] = {c->grid.nx, c->grid.ny, c->grid.nz};
  int rc0 = stage64(si, st);
  if (rc0 != X3D_OK) return rc0;
  // 9 first + 9 second derivatives in FP64 (postprocess_tgv), in FP64 buffers
  std::vector<double*> g(9), l(9);
  double* buf = nullptr;
  if (cudaMalloc(&buf, (size_t)18 * si->N * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
  for (int q = 0; q < 9; ++q) { g[q] = buf + (size_t)q * si->N; l[q] = buf + (size_t)(9 + q) * si->N; }
  const double* u[3] = {si->ux, si->uy, si->uz};
  // parity as in src/Case-TGV.f90:246-264: d(u)/dx odd(0), d(v)/dx even(1), ...
  const int par1[3][3] = {{0, 1, 1}, {1, 0, 1}, {1, 1, 0}};  // [axis][component]
  int rc = X3D_OK;
  for (int a = 0; a < 3 && rc == X3D_OK; ++a)
    for (int q = 0; q < 3 && rc == X3D_OK; ++q) {
      OpPlan* p1 = nullptr;
      OpPlan* p2 = nullptr;
      const int np = par1[a][q];
      rc = get_plan(c, a, K_DER1, np, default_coefset(K_DER1, np), &p1);
      if (rc == X3D_OK) rc = get_plan(c, a, K_DER2, np, default_coefset(K_DER2, np), &p2);
      if (rc == X3D_OK) rc = launch_line_op<double>(c, p1, g[a * 3 + q], u[q], dims, nullptr, st);
      if (rc == X3D_OK) rc = launch_line_op<double>(c, p2, l[a * 3 + q], u[q], dims, nullptr, st);
    }
  if (rc == X3D_OK) {
    double** dg = nullptr;
    cudaMalloc(&dg, 18 * sizeof(double*));
    std::vector<double*> all(g);
    all.insert(all.end(), l.begin(), l.end());
    cudaMemcpyAsync(dg, all.data(), 18 * sizeof(double*), cudaMemcpyHostToDevice, st);
    const unsigned nb = std::min<unsigned>(4096, pw_blocks(c, si->N));
    // statistics over the reference's points: nxc = nxm on a free-slip axis
    int sub[3];
    double nc = 1.0;
    for (int a = 0; a < 3; ++a) {
      const bool fs = (c->ax[a].ncl1 == 1);
      sub[a] = fs ? dims[a] - 1 : dims[a];
      nc *= fs ? (double)c->ax[a].nm : (double)dims[a];
    }
    k_stats<<<nb, 256, 0, st>>>(si->ux, si->uy, si->uz, dg, dg + 9, si->o.xnu, si->N, dims[0], dims[1], sub[0],
                                sub[1], sub[2], si->part);
    cudaMemcpyAsync(si->hpart, si->part, (size_t)nb * 4 * sizeof(double), cudaMemcpyDeviceToHost, st);
    rc = cuda_status(cudaStreamSynchronize(st));
    double acc[4] = {0, 0, 0, 0};
    for (unsigned b = 0; b < nb; ++b)
      for (int q = 0; q < 4; ++q) acc[q] += si->hpart[(size_t)b * 4 + q];
    out[0] = acc[0] / nc;
    out[1] = acc[1] / nc;
    out[2] = acc[3] / nc;
    out[3] = acc[2] / nc;
    cudaFree(dg);
  }
  cudaFree(buf);
  return rc;
}

int x3d_solver_divmax(x3d_solver* s, double* out, void* stream) {
  if (!s || !out) return X3D_ERR_ARG;
  SolverImpl* si = &s->impl;
  xfer_drain(si);
  Ctx* c = si->c;
  cudaStream_t st = (cudaStream_t)stream;
  int rc0 = stage64(si, st);
  if (rc0 != X3D_OK) return rc0;
  // always evaluated in FP64 on the FP64 state
  double* tmp = nullptr;
  double* P[7];
  if (cudaMalloc(&tmp, (size_t)8 * si->N * sizeof(double)) != cudaSuccess) return X3D_ERR_NOMEM;
  for (int k = 0; k < 7; ++k) P[k] = tmp + (size_t)k * si->N;
  void* saveP[8];
  std::memcpy(saveP, si->P, sizeof(saveP));
  for (int k = 0; k < 7; ++k) si->P[k] = P[k];
  double* dv = tmp + (size_t)7 * si->N;
  int rc = divergence<double>(si, si->ux, si->uy, si->uz, dv, true, st);
  std::memcpy(si->P, saveP, sizeof(saveP));
  if (rc == X3D_OK) {
    const unsigned nb = std::min<unsigned>(4096, pw_blocks(c, si->Np));
    k_absmax<<<nb, 256, 0, st>>>(dv, si->Np, si->part);
    cudaMemcpyAsync(si->hpart, si->part, nb * sizeof(double), cudaMemcpyDeviceToHost, st);
    rc = cuda_status(cudaStreamSynchronize(st));
    double m = 0;
    for (unsigned b = 0; b < nb; ++b) m = std::max(m, si->hpart[b]);
    *out = m;
  }
  cudaFree(tmp);
  return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Stand-alone projection pieces (C ABI), FP64, on context scratch.
// ---------------------------------------------------------------------------
extern "C" {

int x3d_divergence(x3d_ctx* h, double* pp3, const double* ux, const double* uy, const double* uz, void* stream) {
  if (!h || !pp3 || !ux || !uy || !uz) return X3D_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  SolverImpl s;
  s.c = c;
  s.N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
  s.Np = (long long)c->ax[0].nm * c->ax[1].nm * c->ax[2].nm;
  void* ws = nullptr;
  int rc = ctx_workspace(c, (size_t)7 * s.N * sizeof(double), &ws);
  if (rc != X3D_OK) return rc;
  for (int k = 0; k < 7; ++k) s.P[k] = (double*)ws + (size_t)k * s.N;
  return divergence<double>(&s, ux, uy, uz, pp3, true, (cudaStream_t)stream);
}

int x3d_gradp(x3d_ctx* h, double* px, double* py, double* pz, const double* pp3, void* stream) {
  if (!h || !px || !py || !pz || !pp3) return X3D_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  SolverImpl s;
  s.c = c;
  s.N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
  void* ws = nullptr;
  int rc = ctx_workspace(c, (size_t)5 * s.N * sizeof(double), &ws);
  if (rc != X3D_OK) return rc;
  for (int k = 0; k < 5; ++k) s.P[k] = (double*)ws + (size_t)k * s.N;
  return gradp<double>(&s, pp3, px, py, pz, (cudaStream_t)stream);
}

int x3d_divergence_f32(x3d_ctx* h, double* pp3, const float* ux, const float* uy, const float* uz, void* stream) {
  if (!h || !pp3 || !ux || !uy || !uz) return X3D_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (c->st.istret != 0) return X3D_ERR_UNSUPPORTED;
  SolverImpl s;
  s.c = c;
  s.N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
  s.Np = (long long)c->ax[0].nm * c->ax[1].nm * c->ax[2].nm;
  void* ws = nullptr;
  int rc = ctx_workspace(c, (size_t)7 * s.N * sizeof(float), &ws);
  if (rc != X3D_OK) return rc;
  for (int k = 0; k < 7; ++k) s.P[k] = (float*)ws + (size_t)k * s.N;
  return divergence<float>(&s, ux, uy, uz, pp3, true, (cudaStream_t)stream);
}

int x3d_gradp_f32(x3d_ctx* h, float* px, float* py, float* pz, const float* pp3, void* stream) {
  if (!h || !px || !py || !pz || !pp3) return X3D_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (c->st.istret != 0) return X3D_ERR_UNSUPPORTED;
  SolverImpl s;
  s.c = c;
  s.N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
  void* ws = nullptr;
  int rc = ctx_workspace(c, (size_t)5 * s.N * sizeof(float), &ws);
  if (rc != X3D_OK) return rc;
  for (int k = 0; k < 5; ++k) s.P[k] = (float*)ws + (size_t)k * s.N;
  return gradp<float>(&s, pp3, px, py, pz, (cudaStream_t)stream);
}

int x3d_cor_vel(x3d_ctx* h, double* ux, double* uy, double* uz, const double* px, const double* py,
                const double* pz, void* stream) {
  if (!h || !ux || !uy || !uz || !px || !py || !pz) return X3D_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  const long long N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
  k_corvel<double><<<pw_blocks(c, N), 256, 0, (cudaStream_t)stream>>>(ux, uy, uz, px, py, pz, N);
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
