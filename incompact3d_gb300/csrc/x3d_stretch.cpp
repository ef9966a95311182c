// Host-side tables of the stretched / non-periodic y direction:
//   * mesh stretching metrics (src/stretching.f90:92-270, stretching_full) and
//     the uniform-mesh defaults of src/variables.f90:1294-1305;
//   * the wavenumber, transfer-function and shift tables poisson_010 needs for
//     a non-periodic y axis (src/poisson.f90:1489-1496 abxyz, 1603-1619 and
//     1663-1676 waves).
// Expressions keep the reference's operation order so the tables match the
// Fortran values to the last bit on the same libm.
#include <cmath>

#include "x3d_internal.h"

namespace x3d {

namespace {
const double kPi = std::acos(-1.0);
}

int build_stretch(const x3d_grid& g, const AxisCoef& a, Stretch& st) {
  const int ny = g.ny;
  const double PI = kPi, yly = g.yly;
  st.istret = g.istret;
  st.beta = g.beta;
  st.alpha = 0;
  st.yp.assign(ny, 0.0); st.ypi.assign(ny, 0.0);
  st.ppy.assign(ny, 1.0); st.pp2y.assign(ny, 0.0); st.pp4y.assign(ny, 0.0);
  st.ppyi.assign(ny, 1.0); st.pp2yi.assign(ny, 0.0); st.pp4yi.assign(ny, 0.0);
  if (g.istret == 0) {
    for (int j = 0; j < ny; ++j) {
      st.yp[j] = (double)j * a.d;
      st.ypi[j] = ((double)(j + 1) - 0.5) * a.d;
    }
    if (a.ncl1 == 1 || a.ncl1 == 2) st.ppy[0] = 2.0;
    if (a.ncln == 1 || a.ncln == 2) st.ppy[ny - 1] = 2.0;
    return X3D_OK;
  }
  if (g.istret < 0 || g.istret > 3) return X3D_ERR_UNSUPPORTED;
  if (a.periodic) return X3D_ERR_BC;  // stretching needs a non-periodic y (src/parameters.f90:283)
  if (!(g.beta > 0)) return X3D_ERR_ARG;
  const int istret = g.istret;
  const double beta = g.beta;
  const int nym = ny - 1;
  const double yinf = -yly / 2.0;
  const double den = 2.0 * beta * yinf;
  const double xnum = -yinf - std::sqrt(PI * PI * beta * beta + yinf * yinf);
  const double alpha = std::fabs(xnum / den);
  st.alpha = alpha;
  // physical coordinate of the computational coordinate ye
  auto map = [&](double ye) {
    const double den1 = std::sqrt(alpha * beta + 1.0);
    const double xn = den1 / std::sqrt(alpha / PI) / std::sqrt(beta) / std::sqrt(PI);
    const double dn = 2.0 * std::sqrt(alpha / PI) * std::sqrt(beta) * PI * std::sqrt(PI);
    const double den3 = ((std::sin(PI * ye)) * (std::sin(PI * ye)) / beta / PI) + alpha / PI;
    const double den4 = 2.0 * alpha * beta - std::cos(2.0 * PI * ye) + 1.0;
    const double xnum1 = (std::atan(xn * std::tan(PI * ye))) * den4 / den1 / den3 / dn;
    const double cst = std::sqrt(beta) * PI / (2.0 * std::sqrt(alpha) * std::sqrt(alpha * beta + 1.0));
    const double off = (istret == 1) ? -yinf : yly;
    double y = 0.0;
    if (ye < 0.5) y = xnum1 - cst + off;
    if (ye == 0.5) y = 0.0 + off;
    if (ye > 0.5) y = xnum1 + cst + off;
    return (istret == 3) ? y * 2.0 : y;
  };
  dvec yeta(ny, 0.0), yetai(ny, 0.0);
  yeta[0] = (istret == 1) ? 0.0 : -0.5;
  st.yp[0] = 0.0;
  for (int j = 2; j <= ny; ++j) {
    if (istret == 1) yeta[j - 1] = (double)(j - 1) * (1.0 / (double)nym);
    if (istret == 2) yeta[j - 1] = (double)(j - 1) * (1.0 / (double)nym) - 0.5;
    if (istret == 3) yeta[j - 1] = (double)(j - 1) * (0.5 / (double)nym) - 0.5;
    st.yp[j - 1] = map(yeta[j - 1]);
  }
  for (int j = 1; j <= ny; ++j) {
    if (istret == 1) yetai[j - 1] = ((double)j - 0.5) * (1.0 / (double)nym);
    if (istret == 2) yetai[j - 1] = ((double)j - 0.5) * (1.0 / (double)nym) - 0.5;
    if (istret == 3) yetai[j - 1] = ((double)j - 0.5) * (0.5 / (double)nym) - 0.5;
    st.ypi[j - 1] = map(yetai[j - 1]);
  }
  for (int j = 0; j < ny; ++j) {
    st.ppy[j] = yly * (alpha / PI + (1.0 / PI / beta) * std::sin(PI * yeta[j]) * std::sin(PI * yeta[j]));
    st.pp2y[j] = st.ppy[j] * st.ppy[j];
    st.pp4y[j] = (-2.0 / beta * std::cos(PI * yeta[j]) * std::sin(PI * yeta[j]));
    st.ppyi[j] = yly * (alpha / PI + (1.0 / PI / beta) * std::sin(PI * yetai[j]) * std::sin(PI * yetai[j]));
    st.pp2yi[j] = st.ppyi[j] * st.ppyi[j];
    st.pp4yi[j] = (-2.0 / beta * std::cos(PI * yetai[j]) * std::sin(PI * yetai[j]));
    if (istret == 3) {
      st.pp4y[j] = st.pp4y[j] / 2.0;
      st.pp4yi[j] = st.pp4yi[j] / 2.0;
    }
  }
  return X3D_OK;
}

void waves_y010(const AxisCoef& a, int istret, double yly, dvec& yky, dvec& yk2, dvec& tr, dvec& sa, dvec& sb) {
  const int ny = a.n, nym = a.nm;
  const double PI = kPi, twopi = 2.0 * kPi;
  yky.assign(ny, 0.0);
  yk2.assign(ny, 0.0);
  dvec eys(ny, 0.0);
  for (int j = 1; j <= ny; ++j) {
    const double w = twopi * 0.5 * (double)(j - 1) / (double)nym;
    double wp = a.aci6 * 2.0 * a.d * std::sin(w * 0.5) + (a.bci6 * 2.0 * a.d) * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * a.alcai6 * std::cos(w));
    yky[j - 1] = (istret == 0) ? (double)nym * wp / yly : (double)nym * wp;
    eys[j - 1] = (double)nym * w / yly;
    const double t = (double)nym * wp / yly;
    yk2[j - 1] = t * t;
  }
  yky[0] = 0.0;
  eys[0] = 0.0;
  yk2[0] = 0.0;
  tr.assign(nym, 0.0);
  for (int j = 0; j < nym; ++j) {
    const double rl = eys[j] * a.d;
    const double tt = 2.0 * (a.bici6 * std::cos(rl * 1.5) + a.cici6s * std::cos(rl * 2.5) + a.dici6 * std::cos(rl * 3.5));
    const double tt1 = 2.0 * a.aici6 * std::cos(rl * 0.5);
    const double t1 = 1.0 + 2.0 * a.ailcai6 * std::cos(rl);
    tr[j] = (tt1 + tt) / t1;
  }
  sa.assign(nym, 0.0);
  sb.assign(nym, 0.0);
  for (int j = 1; j <= nym; ++j) {
    sa[j - 1] = std::sin((double)(j - 1) * PI * 0.5 / (double)nym);
    sb[j - 1] = std::cos((double)(j - 1) * PI * 0.5 / (double)nym);
  }
}

}  // namespace x3d
