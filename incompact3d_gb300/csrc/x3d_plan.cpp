// Host-side setup of libx3dgpu: the compact-scheme coefficients, their Thomas
// factorisations, and per-operator plans (interior stencil, boundary-row
// tables, Sherman-Morrison vector, chunked-solve fix-up factors).
//
// The coefficient values restate the reference's init-time routines:
//   prepare              src/schemes.f90:413-439
//   first_derivative     src/schemes.f90:443-599
//   second_derivative    src/schemes.f90:602-856
//   interpolation        src/schemes.f90:860-1066
//   set_filter_coefficients  src/filters.f90:62-219
//   waves (periodic)     src/poisson.f90:1530-1810
// and are bit-compatible with them (same operations in the same order).
#include <cmath>
#include <cstring>

#include "x3d_internal.h"

namespace x3d {

namespace {

// LU factors of the tridiagonal (lower b, diagonal c, upper f), in the form
// the sweeps consume: s(i) = b(i-1)/w(i-1), w = 1/pivot.
void factor(const dvec& b, const dvec& c, const dvec& f, dvec& s, dvec& w) {
  const size_t n = c.size();
  s.assign(n, 0.0);
  w = c;
  for (size_t i = 1; i < n; ++i) {
    s[i] = b[i - 1] / w[i - 1];
    w[i] = w[i] - f[i - 1] * s[i];
  }
  for (size_t i = 0; i < n; ++i) w[i] = 1.0 / w[i];
}

// Diagonals of a collocated scheme with constant interior alpha and `nb`
// boundary rows at each end; rows near the ends are overwritten by the caller.
struct Tri {
  dvec b, c, f;
  explicit Tri(int n, double al) : b(n, al), c(n, 1.0), f(n, al) {}
};

void set3(dvec* v, int idx, double x) { (*v)[idx] = x; }

}  // namespace

int build_axis(AxisCoef& a, int n, double len, int ncl1, int ncln, const x3d_numopts& o) {
  if (n < 8) return X3D_ERR_SHAPE;
  if (ncl1 < 0 || ncl1 > 2 || ncln < 0 || ncln > 2) return X3D_ERR_BC;
  if ((ncl1 == 0) != (ncln == 0)) return X3D_ERR_BC;
  if (o.ifirstder != 1 && o.ifirstder != 4) return X3D_ERR_UNSUPPORTED;
  if (o.isecondder != 1 && o.isecondder != 4 && o.isecondder != 5) return X3D_ERR_UNSUPPORTED;
  if (o.ipinter < 1 || o.ipinter > 3) return X3D_ERR_UNSUPPORTED;
  a.n = n;
  a.ncl1 = ncl1;
  a.ncln = ncln;
  a.periodic = (ncl1 == 0);
  a.nm = a.periodic ? n : n - 1;
  a.len = len;
  a.d = len / (double)a.nm;  // src/parameters.f90:296-298
  a.d2 = a.d * a.d;
  const double d = a.d, d2 = a.d2;
  dvec* V = a.vecs;

  // ---- first derivative ---------------------------------------------------
  if (o.ifirstder == 1) {
    a.alfai = 0.0; a.afi = 1.0 / (2.0 * d); a.bfi = 0.0;
    a.alfa1 = a.af1 = a.bf1 = a.cf1 = a.alfa2 = a.af2 = 0.0;
    a.alfam = a.afm = a.alfan = a.afn = a.bfn = a.cfn = 0.0;
  } else {
    a.alfai = 1.0 / 3.0; a.afi = (7.0 / 9.0) / d; a.bfi = (1.0 / 36.0) / d;
    a.alfa1 = 2.0; a.af1 = -(5.0 / 2.0) / d; a.bf1 = 2.0 / d; a.cf1 = 0.5 / d;
    a.alfa2 = 1.0 / 4.0; a.af2 = (3.0 / 4.0) / d;
    a.alfan = 2.0; a.afn = -(5.0 / 2.0) / d; a.bfn = 2.0 / d; a.cfn = 0.5 / d;
    a.alfam = 1.0 / 4.0; a.afm = (3.0 / 4.0) / d;
  }
  {
    const double al = a.alfai;
    Tri t(n, al);
    t.c[0] = (ncl1 == 0) ? 2.0 : 1.0;
    if (ncl1 == 1) t.f[0] = al + al;
    if (ncl1 == 2) { t.f[0] = a.alfa1; t.f[1] = a.alfa2; t.b[0] = a.alfa2; }
    t.f[n - 1] = 0.0; t.b[n - 1] = 0.0;
    if (ncln == 0) t.c[n - 1] = 1.0 + al * al;
    if (ncln == 1) t.b[n - 2] = al + al;
    if (ncln == 2) { t.f[n - 2] = a.alfam; t.b[n - 3] = a.alfam; t.b[n - 2] = a.alfan; }
    dvec fp = t.f;
    V[X3D_COEF_FF] = t.f;
    factor(t.b, t.c, t.f, V[X3D_COEF_FS], V[X3D_COEF_FW]);
    if (ncl1 == 1) fp[0] = 0.0;
    if (ncln == 1) t.b[n - 2] = 0.0;
    V[X3D_COEF_FFP] = fp;
    factor(t.b, t.c, fp, V[X3D_COEF_FSP], V[X3D_COEF_FWP]);
  }

  // ---- second derivative --------------------------------------------------
  if (o.isecondder == 1) {
    a.alsai = 0; a.asi = 1.0 / d2; a.bsi = 0; a.csi = 0; a.dsi = 0;
  } else if (o.isecondder == 4) {
    a.alsai = 2.0 / 11.0; a.asi = (12.0 / 11.0) / d2; a.bsi = (3.0 / 44.0) / d2; a.csi = 0; a.dsi = 0;
  } else {
    const double pi = std::acos(-1.0);
    const double dpis3 = 2.0 * pi / 3.0;
    const double xnpi2 = pi * pi * (1.0 + o.nu0nu);
    const double xmpi2 = dpis3 * dpis3 * (1.0 + o.cnu * o.nu0nu);
    const double den = 405.0 * xnpi2 - 640.0 * xmpi2 + 144.0;
    a.alsai = 0.5 - (320.0 * xmpi2 - 1296.0) / den;
    a.asi = -(4329.0 * xnpi2 / 8.0 - 32.0 * xmpi2 - 140.0 * xnpi2 * xmpi2 + 286.0) / den / d2;
    a.bsi = (2115.0 * xnpi2 - 1792.0 * xmpi2 - 280.0 * xnpi2 * xmpi2 + 1328.0) / den / (4.0 * d2);
    a.csi = -(7695.0 * xnpi2 / 8.0 + 288.0 * xmpi2 - 180.0 * xnpi2 * xmpi2 - 2574.0) / den / (9.0 * d2);
    a.dsi = (198.0 * xnpi2 + 128.0 * xmpi2 - 40.0 * xnpi2 * xmpi2 - 736.0) / den / (16.0 * d2);
  }
  a.as1 = 13.0 / d2; a.bs1 = -27.0 / d2; a.cs1 = 15.0 / d2; a.ds1 = -1.0 / d2;
  a.asn = a.as1; a.bsn = a.bs1; a.csn = a.cs1; a.dsn = a.ds1;
  const double alsa2 = (o.isecondder == 1) ? 0.0 : 0.1;
  a.as2 = (o.isecondder == 1) ? 1.0 / d2 : (6.0 / 5.0) / d2;
  a.asm_ = a.as2;
  a.as3 = (12.0 / 11.0) / d2; a.bs3 = (3.0 / 44.0) / d2;
  a.as4 = a.as3; a.bs4 = a.bs3; a.cs4 = 0.0;
  a.ast = a.as3; a.bst = a.bs3;
  a.astt = a.as3; a.bstt = a.bs3; a.cstt = 0.0;
  {
    const double al = a.alsai;
    const double a34 = 2.0 / 11.0;  // alsa3 = alsa4 = alsat = alsatt
    Tri t(n, al);
    if (ncl1 == 0) t.c[0] = 2.0;
    if (ncl1 == 1) t.f[0] = al + al;
    if (ncl1 == 2) {
      t.f[0] = 11.0; t.f[1] = alsa2; t.f[2] = a34; t.f[3] = a34;
      t.b[0] = alsa2; t.b[1] = a34; t.b[2] = a34; t.b[3] = al;
    }
    // right-end rows n-5..n-1 are (re)assigned after the left ones, as in
    // the reference; on an 8-point line they overlap the left rows.
    for (int i = n - 5; i < n - 1; ++i) { t.f[i] = al; t.c[i] = 1.0; t.b[i] = al; }
    t.f[n - 1] = 0.0; t.b[n - 1] = 0.0; t.c[n - 1] = 1.0;
    if (ncln == 0) t.c[n - 1] = 1.0 + al * al;
    if (ncln == 1) t.b[n - 2] = al + al;
    if (ncln == 2) {
      t.f[n - 4] = a34; t.f[n - 3] = a34; t.f[n - 2] = alsa2;
      t.b[n - 5] = a34; t.b[n - 4] = a34; t.b[n - 3] = alsa2; t.b[n - 2] = 11.0;
    }
    dvec fp = t.f;
    dvec fpl = t.f;
    if (ncl1 == 1) fpl[0] = 0.0;
    V[X3D_COEF_SFP] = fp;
    V[X3D_COEF_SF] = fpl;
    factor(t.b, t.c, fp, V[X3D_COEF_SSP], V[X3D_COEF_SWP]);
    if (ncln == 1) t.b[n - 2] = 0.0;
    factor(t.b, t.c, fpl, V[X3D_COEF_SS], V[X3D_COEF_SW]);
  }

  // ---- staggered derivative / interpolation -------------------------------
  if (o.ifirstder == 1) {
    a.alcai6 = 0.0; a.aci6 = 1.0 / d; a.bci6 = 0.0;
    a.ailcai6 = 0.0; a.aici6 = 0.5; a.bici6 = 0.0; a.cici6s = 0.0; a.dici6 = 0.0;
  } else {
    a.alcai6 = 9.0 / 62.0; a.aci6 = (63.0 / 62.0) / d; a.bci6 = (17.0 / 62.0) / 3.0 / d;
    if (o.ipinter == 1) {
      a.ailcai6 = 3.0 / 10.0; a.aici6 = 3.0 / 4.0; a.bici6 = 1.0 / (2.0 * 10.0); a.cici6s = 0.0; a.dici6 = 0.0;
    } else if (o.ipinter == 2) {
      a.ailcai6 = 0.461658;
      a.dici6 = 0.00293016;
      a.aici6 = 1.0 / 64.0 * (75.0 + 70.0 * a.ailcai6 - 320.0 * a.dici6);
      a.bici6 = 1.0 / 128.0 * (126.0 * a.ailcai6 - 25.0 + 1152.0 * a.dici6);
      a.cici6s = 1.0 / 128.0 * (-10.0 * a.ailcai6 + 3.0 - 640.0 * a.dici6);
      a.aici6 /= 2.0; a.bici6 /= 2.0; a.cici6s /= 2.0; a.dici6 /= 2.0;
    } else {
      a.ailcai6 = 0.49;
      a.aici6 = 1.0 / 128.0 * (75.0 + 70.0 * a.ailcai6);
      a.bici6 = 1.0 / 256.0 * (126.0 * a.ailcai6 - 25.0);
      a.cici6s = 1.0 / 256.0 * (-10.0 * a.ailcai6 + 3.0);
      a.dici6 = 0.0;
    }
  }
  {
    const int nm = a.nm;
    // pressure-mesh diagonals (length nm)
    auto pmesh = [&](double al, dvec& b, dvec& c, dvec& f) {
      b.assign(nm, al); c.assign(nm, 1.0); f.assign(nm, al);
      f[nm - 1] = 0.0; b[nm - 1] = 0.0;
      c[0] = (ncl1 == 0) ? 2.0 : 1.0 + al;
      c[nm - 1] = (ncln == 0) ? 1.0 + al * al : 1.0 + al;
    };
    // velocity-mesh diagonals (length n) used by the non-periodic p->v operators
    auto vmesh = [&](double al, dvec& b, dvec& c, dvec& f) {
      b.assign(n, al); c.assign(n, 1.0); f.assign(n, al);
      f[0] = al + al; f[n - 1] = 0.0;
      b[n - 2] = al + al; b[n - 1] = 0.0;
    };
    dvec cb, cc, cf, cib, cic, cif, bi, ci, fi, ibi, ici, ifi;
    pmesh(a.alcai6, cb, cc, cf);
    pmesh(a.ailcai6, cib, cic, cif);
    vmesh(a.alcai6, bi, ci, fi);
    vmesh(a.ailcai6, ibi, ici, ifi);
    dvec cfp = cf, cifp = cif, cfip = fi, cifip = ifi;
    cfp[0] = 0.0;
    cfip[0] = 0.0;
    V[X3D_COEF_CF6] = cf;   factor(cb, cc, cf, V[X3D_COEF_CS6], V[X3D_COEF_CW6]);
    V[X3D_COEF_CIF6] = cif; factor(cib, cic, cif, V[X3D_COEF_CIS6], V[X3D_COEF_CIW6]);
    V[X3D_COEF_CFI6] = fi;  factor(bi, ci, fi, V[X3D_COEF_CSI6], V[X3D_COEF_CWI6]);
    V[X3D_COEF_CIFI6] = ifi; factor(ibi, ici, ifi, V[X3D_COEF_CISI6], V[X3D_COEF_CIWI6]);
    if (ncln != 0) {
      cb[nm - 2] = 0.0; cib[nm - 1] = 0.0; bi[n - 2] = 0.0; ibi[n - 1] = 0.0;
    }
    V[X3D_COEF_CFP6] = cfp;    factor(cb, cc, cfp, V[X3D_COEF_CSP6], V[X3D_COEF_CWP6]);
    V[X3D_COEF_CIFP6] = cifp;  factor(cib, cic, cifp, V[X3D_COEF_CISP6], V[X3D_COEF_CIWP6]);
    V[X3D_COEF_CFIP6] = cfip;  factor(bi, ci, cfip, V[X3D_COEF_CSIP6], V[X3D_COEF_CWIP6]);
    V[X3D_COEF_CIFIP6] = cifip; factor(ibi, ici, cifip, V[X3D_COEF_CISIP6], V[X3D_COEF_CIWIP6]);
  }

  // ---- filter ------------------------------------------------------------
  {
    const double af = o.filter_alpha;
    a.fiali = af;
    a.fiai = (11.0 + 10.0 * af) / 16.0;
    a.fibi = 0.5 * (15.0 + 34.0 * af) / 32.0;
    a.fici = 0.5 * (-3.0 + 6.0 * af) / 16.0;
    a.fidi = 0.5 * (1.0 - 2.0 * af) / 32.0;
    a.fia2 = 1.0 / 8.0 + 3.0 / 4.0 * af; a.fib2 = 5.0 / 8.0 + 3.0 / 4.0 * af;
    a.fic2 = 3.0 / 8.0 + af / 4.0; a.fid2 = -1.0 / 8.0 + af / 4.0;
    a.fia3 = -1.0 / 32.0 + af / 16.0; a.fib3 = 5.0 / 32.0 + 11.0 / 16.0 * af;
    a.fic3 = 11.0 / 16.0 + 5.0 * af / 8.0; a.fid3 = 5.0 / 16.0 + 3.0 * af / 8.0;
    a.fie3 = -5.0 / 32.0 + 5.0 * af / 16.0; a.fif3 = 1.0 / 32.0 - af / 16.0;
    a.fiam = a.fia2; a.fibm = a.fib2; a.ficm = a.fic2; a.fidm = a.fid2;
    a.fiap = a.fia3; a.fibp = a.fib3; a.ficp = a.fic3; a.fidp = a.fid3; a.fiep = a.fie3; a.fifp = a.fif3;
    Tri t(n, af);
    t.c[0] = (ncl1 == 0) ? 2.0 : 1.0;
    if (ncl1 == 1) t.f[0] = af + af;
    if (ncl1 == 2) { t.f[0] = 0.0; t.f[1] = af; t.b[0] = af; }  // alfa1 = 0, alfa2 = af
    t.f[n - 1] = 0.0; t.b[n - 1] = 0.0;
    if (ncln == 0) t.c[n - 1] = 1.0 + af * af;
    if (ncln == 1) t.b[n - 2] = af + af;
    if (ncln == 2) { t.f[n - 2] = af; t.b[n - 3] = af; t.b[n - 2] = 0.0; }  // alfam = af, alfan = 0
    dvec fp = t.f;
    V[X3D_COEF_FIFFP] = fp;
    factor(t.b, t.c, fp, V[X3D_COEF_FIFSP], V[X3D_COEF_FIFWP]);
    if (ncl1 == 1) t.f[0] = 0.0;
    if (ncln == 1) t.b[n - 2] = 0.0;
    V[X3D_COEF_FIFF] = t.f;
    factor(t.b, t.c, t.f, V[X3D_COEF_FIFS], V[X3D_COEF_FIFW]);
  }
  (void)set3;
  return X3D_OK;
}

int default_coefset(int kind, int npaire) {
  (void)kind;
  return npaire == 1 ? 1 : 0;
}

void coef_indices(const AxisCoef& a, int kind, int coefset, int* fi, int* si, int* wi) {
  int base = 0;
  switch (kind) {
    case K_DER1: base = coefset ? X3D_COEF_FFP : X3D_COEF_FF; break;
    case K_DER2: base = coefset ? X3D_COEF_SFP : X3D_COEF_SF; break;
    case K_FIL: base = coefset ? X3D_COEF_FIFFP : X3D_COEF_FIFF; break;
    case K_DVP: base = coefset ? X3D_COEF_CFP6 : X3D_COEF_CF6; break;
    case K_IVP: base = coefset ? X3D_COEF_CIFP6 : X3D_COEF_CIF6; break;
    case K_DPV: base = a.periodic ? X3D_COEF_CF6 : (coefset ? X3D_COEF_CFIP6 : X3D_COEF_CFI6); break;
    case K_IPV: base = a.periodic ? X3D_COEF_CIF6 : (coefset ? X3D_COEF_CIFIP6 : X3D_COEF_CIFI6); break;
  }
  *fi = base;
  *si = base + 1;
  *wi = base + 2;
}

namespace {

struct Ent { int mult; int idx; };
struct Term { double coef; std::vector<Ent> e; };
typedef std::vector<Term> Expr;

// Interior stencil of each kind at output row r, term by term in the order the
// reference writes it (relative input indices).
Expr interior(int kind, int r, double ca, double cb, double cc, double cd) {
  switch (kind) {
    case K_DER1:
      return {{ca, {{1, r + 1}, {-1, r - 1}}}, {cb, {{1, r + 2}, {-1, r - 2}}}};
    case K_DER2:
      return {{ca, {{1, r + 1}, {-1, r}, {-1, r}, {1, r - 1}}},
              {cb, {{1, r + 2}, {-1, r}, {-1, r}, {1, r - 2}}},
              {cc, {{1, r + 3}, {-1, r}, {-1, r}, {1, r - 3}}},
              {cd, {{1, r + 4}, {-1, r}, {-1, r}, {1, r - 4}}}};
    case K_FIL:
      return {{ca, {{1, r}}}, {cb, {{1, r + 1}, {1, r - 1}}}, {cc, {{1, r + 2}, {1, r - 2}}},
              {cd, {{1, r + 3}, {1, r - 3}}}};
    case K_DVP:
      return {{ca, {{1, r + 1}, {-1, r}}}, {cb, {{1, r + 2}, {-1, r - 1}}}};
    case K_IVP:
      return {{ca, {{1, r + 1}, {1, r}}}, {cb, {{1, r + 2}, {1, r - 1}}}, {cc, {{1, r + 3}, {1, r - 2}}},
              {cd, {{1, r + 4}, {1, r - 3}}}};
    case K_DPV:
      return {{ca, {{1, r}, {-1, r - 1}}}, {cb, {{1, r + 1}, {-1, r - 2}}}};
    case K_IPV:
    default:
      return {{ca, {{1, r}, {1, r - 1}}}, {cb, {{1, r + 1}, {1, r - 2}}}, {cc, {{1, r + 2}, {1, r - 3}}},
              {cd, {{1, r + 3}, {1, r - 4}}}};
  }
}

void stencil_extent(int kind, int* lo, int* hi) {
  static const int L[K_COUNT] = {-2, -4, -3, -1, -3, -2, -4};
  static const int H[K_COUNT] = {2, 4, 3, 2, 4, 1, 3};
  *lo = L[kind];
  *hi = H[kind];
}

Term one(double coef, int idx) { return Term{coef, {{1, idx}}}; }

// Explicit one-sided rows of the Dirichlet (ncl=2) closures.
// left=true: rows 0.. of the line; indices absolute.  n = line length.
bool dirichlet_row(const AxisCoef& a, int kind, bool left, int r, int n, Expr* out) {
  Expr& e = *out;
  e.clear();
  auto D2 = [](double c, int ip, int i, int im) { return Term{c, {{1, ip}, {-1, i}, {-1, i}, {1, im}}}; };
  if (kind == K_DER1) {  // src/derive.f90:211-321 (derx_21/12/22)
    if (left) {
      if (r == 0) e = {one(a.af1, 0), one(a.bf1, 1), one(a.cf1, 2)};
      else if (r == 1) e = {Term{a.af2, {{1, 2}, {-1, 0}}}};
      else return false;
    } else {
      if (r == n - 2) e = {Term{a.afm, {{1, n - 1}, {-1, n - 3}}}};
      else if (r == n - 1) e = {one(-a.afn, n - 1), one(-a.bfn, n - 2), one(-a.cfn, n - 3)};
      else return false;
    }
    return true;
  }
  if (kind == K_DER2) {  // src/derive.f90:1666-2048 (derxx_12/21/22)
    if (left) {
      if (r == 0) e = {one(a.as1, 0), one(a.bs1, 1), one(a.cs1, 2), one(a.ds1, 3)};
      else if (r == 1) e = {D2(a.as2, 2, 1, 0)};
      else if (r == 2) e = {D2(a.as3, 3, 2, 1), D2(a.bs3, 4, 2, 0)};
      else if (r == 3) e = {D2(a.as4, 4, 3, 2), D2(a.bs4, 5, 3, 1), D2(a.cs4, 6, 3, 0)};
      else return false;
    } else {
      if (r == n - 4) e = {D2(a.astt, n - 3, n - 4, n - 5), D2(a.bstt, n - 2, n - 4, n - 6), D2(a.cstt, n - 1, n - 4, n - 7)};
      else if (r == n - 3) e = {D2(a.ast, n - 2, n - 3, n - 4), D2(a.bst, n - 1, n - 3, n - 5)};
      else if (r == n - 2) e = {D2(a.asm_, n - 1, n - 2, n - 3)};
      else if (r == n - 1) e = {one(a.asn, n - 1), one(a.bsn, n - 2), one(a.csn, n - 3), one(a.dsn, n - 4)};
      else return false;
    }
    return true;
  }
  if (kind == K_FIL) {  // src/filters.f90:384-605 (filx_12/21/22)
    if (left) {
      if (r == 0) e = {one(1.0, 0)};
      else if (r == 1) e = {one(a.fia2, 0), one(a.fib2, 1), one(a.fic2, 2), one(a.fid2, 3)};
      else if (r == 2) e = {one(a.fia3, 0), one(a.fib3, 1), one(a.fic3, 2), one(a.fid3, 3), one(a.fie3, 4), one(a.fif3, 5)};
      else return false;
    } else {
      if (r == n - 1) e = {one(1.0, n - 1)};
      else if (r == n - 2) e = {one(a.fiam, n - 1), one(a.fibm, n - 2), one(a.ficm, n - 3), one(a.fidm, n - 4)};
      else if (r == n - 3)
        e = {one(a.fiap, n - 1), one(a.fibp, n - 2), one(a.ficp, n - 3), one(a.fidp, n - 4), one(a.fiep, n - 5), one(a.fifp, n - 6)};
      else return false;
    }
    return true;
  }
  return false;
}

}  // namespace

int build_plan(const AxisCoef& a, int axis, int kind, int npaire, int coefset, OpPlan& p) {
  if (kind < 0 || kind >= K_COUNT || (npaire != 0 && npaire != 1) || (coefset != 0 && coefset != 1))
    return X3D_ERR_ARG;
  p.axis = axis; p.kind = kind; p.npaire = npaire; p.coefset = coefset;
  p.periodic = a.periodic;
  const bool staggered = (kind >= K_DVP);
  const bool vin = !(kind == K_DPV || kind == K_IPV);  // input on the velocity (node) mesh
  p.nin = (kind == K_DPV || kind == K_IPV) ? a.nm : a.n;
  p.nout = (kind == K_DVP || kind == K_IVP) ? a.nm : a.n;
  switch (kind) {
    case K_DER1: p.ca = a.afi; p.cb = a.bfi; p.cc = 0; p.cd = 0; p.alpha = a.alfai; break;
    case K_DER2: p.ca = a.asi; p.cb = a.bsi; p.cc = a.csi; p.cd = a.dsi; p.alpha = a.alsai; break;
    case K_FIL: p.ca = a.fiai; p.cb = a.fibi; p.cc = a.fici; p.cd = a.fidi; p.alpha = a.fiali; break;
    case K_DVP: case K_DPV: p.ca = a.aci6; p.cb = a.bci6; p.cc = 0; p.cd = 0; p.alpha = a.alcai6; break;
    default: p.ca = a.aici6; p.cb = a.bici6; p.cc = a.cici6s; p.cd = a.dici6; p.alpha = a.ailcai6; break;
  }
  // The reference has no non-periodic branch of these three for odd parity.
  if (!a.periodic && npaire == 0 && (kind == K_IVP || kind == K_DPV || kind == K_IPV)) return X3D_ERR_BC;
  int fi, si, wi;
  coef_indices(a, kind, coefset, &fi, &si, &wi);
  p.f = a.vecs[fi];
  p.s = a.vecs[si];
  p.w = a.vecs[wi];
  if ((int)p.f.size() != p.nout) return X3D_ERR_SHAPE;

  // Sherman-Morrison vector r = A^{-1} (-1, 0, ..., 0, alpha), same sweeps as
  // the reference (e.g. src/derive.f90:27-56), and den = 1 + r1 - alpha rn.
  p.rsm.assign(p.nout, 0.0);
  p.nbrows = 0;
  if (a.periodic) {
    const int n = p.nout;
    dvec& r = p.rsm;
    r[0] = -1.0;
    r[n - 1] = p.alpha;
    for (int i = 1; i < n; ++i) r[i] = r[i] - r[i - 1] * p.s[i];
    r[n - 1] = r[n - 1] * p.w[n - 1];
    for (int i = n - 2; i >= 0; --i) r[i] = (r[i] - p.f[i] * r[i + 1]) * p.w[i];
    p.den = 1.0 + r[0] - p.alpha * r[n - 1];
    return X3D_OK;
  }

  // Non-periodic: boundary rows = rows whose interior stencil leaves the line.
  int lo, hi;
  stencil_extent(kind, &lo, &hi);
  const int nin = p.nin, nout = p.nout;
  const int s = (npaire == 1) ? 1 : -1;
  for (int side = 0; side < 2; ++side) {
    const bool left = (side == 0);
    const int ncl = left ? a.ncl1 : a.ncln;
    for (int r = 0; r < nout; ++r) {
      const bool isb = left ? (r + lo < 0) : (r + hi >= nin);
      if (!isb) continue;
      if (left && r + hi >= nin) return X3D_ERR_SHAPE;  // line too short
      Expr e;
      bool done = false;
      if (!staggered && ncl == 2) {
        if (!dirichlet_row(a, kind, left, r, nin, &e)) return X3D_ERR_BC;
        done = true;
      } else if (!staggered && ncl == 1) {
        // free-slip: odd-parity zero rows at the wall node
        const bool wall = left ? (r == 0) : (r == nout - 1);
        if (wall && ((npaire == 0 && (kind == K_DER2 || kind == K_FIL)) || (npaire == 1 && kind == K_DER1))) {
          e.clear();
          done = true;
        }
      } else if (kind == K_DVP && npaire == 0) {
        // src/derive.f90:3875-3880: the odd-parity closure rows of derxvp
        if (left) {
          e = {Term{p.ca, {{1, 1}, {-1, 0}}}, Term{p.cb, {{1, 2}, {-2, 0}, {1, 1}}}};
        } else {
          const int n = nin;
          e = {Term{p.ca, {{1, n - 1}, {-1, n - 2}}}, Term{p.cb, {{2, n - 1}, {-1, n - 2}, {-1, n - 3}}}};
        }
        done = true;
      } else if (kind == K_DPV && npaire == 1) {
        const bool wall = left ? (r == 0) : (r == nout - 1);
        if (wall) { e.clear(); done = true; }
      }
      if (!done) {
        // mirror images across the wall with the parity sign
        e = interior(kind, r, p.ca, p.cb, p.cc, p.cd);
        for (Term& t : e)
          for (Ent& x : t.e) {
            if (x.idx < 0) {
              x.idx = vin ? -x.idx : -1 - x.idx;
              x.mult *= s;
            } else if (x.idx >= nin) {
              x.idx = vin ? 2 * (nin - 1) - x.idx : 2 * nin - 1 - x.idx;
              x.mult *= s;
            }
          }
      }
      if (p.nbrows >= kMaxBRows) return X3D_ERR_UNSUPPORTED;
      BRow& b = p.brows[p.nbrows++];
      b = BRow();
      b.row = r;
      if ((int)e.size() > kMaxTerms) return X3D_ERR_UNSUPPORTED;
      b.nterms = (int)e.size();
      for (size_t t = 0; t < e.size(); ++t) {
        b.coef[t] = e[t].coef;
        if ((int)e[t].e.size() > kMaxEnt) return X3D_ERR_UNSUPPORTED;
        b.nent[t] = (int)e[t].e.size();
        for (size_t q = 0; q < e[t].e.size(); ++q) {
          if (e[t].e[q].idx < 0 || e[t].e[q].idx >= nin) return X3D_ERR_SHAPE;
          b.idx[t][q] = e[t].e[q].idx;
          b.mult[t][q] = e[t].e[q].mult;
        }
      }
    }
  }
  return X3D_OK;
}

void waves_tables(const AxisCoef& a, dvec& k2, dvec& tr) {
  // Periodic branch of src/poisson.f90:1530-1810: modified wavenumber of the
  // staggered first derivative, and the interpolation transfer function that
  // multiplies the other two directions' wavenumbers in kxyz.
  const int n = a.n;
  const double twopi = 2.0 * std::acos(-1.0);
  k2.assign(n, 0.0);
  tr.assign(n, 0.0);
  dvec ex(n, 0.0);
  for (int i = 1; i <= n / 2 + 1; ++i) {
    const double w = twopi * (i - 1) / n;
    double wp = a.aci6 * 2.0 * a.d * std::sin(w * 0.5) + a.bci6 * 2.0 * a.d * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * a.alcai6 * std::cos(w));
    const double kk = n * wp / a.len;
    k2[i - 1] = kk * kk;
    ex[i - 1] = n * w / a.len;
  }
  for (int i = n / 2 + 2; i <= n; ++i) {
    k2[i - 1] = k2[n - i + 1];
    ex[i - 1] = ex[n - i + 1];
  }
  for (int i = 0; i < n; ++i) {
    const double rl = ex[i] * a.d;
    const double tt = 2.0 * (a.bici6 * std::cos(rl * 1.5) + a.cici6s * std::cos(rl * 2.5) + a.dici6 * std::cos(rl * 3.5));
    const double tt1 = 2.0 * a.aici6 * std::cos(rl * 0.5);
    const double t1 = 1.0 + 2.0 * a.ailcai6 * std::cos(rl);
    tr[i] = (tt1 + tt) / t1;
  }
}

// poisson_11x tables (src/poisson.f90:1530-1810 with bcx = bcy = 1, istret = 0):
// the wavenumber^2 and transfer of the modes of a free-slip axis, and kxyz
// as (re, im) per spectral point (i, j, k), i fastest, k < NZ/2+1.  For a
// free-slip z the real part carries mode k and the imaginary part mode NZ-k;
// for a periodic z both parts are equal.
static double transfer_at(const AxisCoef& a, double rl) {
  const double tt = 2.0 * (a.bici6 * std::cos(rl * 1.5) + a.cici6s * std::cos(rl * 2.5) + a.dici6 * std::cos(rl * 3.5));
  const double tt1 = 2.0 * a.aici6 * std::cos(rl * 0.5);
  const double t1 = 1.0 + 2.0 * a.ailcai6 * std::cos(rl);
  return (tt1 + tt) / t1;
}

static void waves_slip(const AxisCoef& a, dvec& k2, dvec& tr) {
  const int nm = a.nm;
  const double twopi = 2.0 * std::acos(-1.0);
  k2.assign(nm, 0.0);
  tr.assign(nm, 0.0);
  dvec es(nm, 0.0);
  for (int i = 1; i <= nm; ++i) {
    const double w = twopi * 0.5 * (double)(i - 1) / (double)nm;
    double wp = a.aci6 * 2.0 * a.d * std::sin(w * 0.5) + (a.bci6 * 2.0 * a.d) * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * a.alcai6 * std::cos(w));
    const double t = (double)nm * wp / a.len;
    k2[i - 1] = t * t;
    es[i - 1] = (double)nm * w / a.len;
  }
  k2[0] = 0.0;
  es[0] = 0.0;
  for (int i = 0; i < nm; ++i) tr[i] = transfer_at(a, es[i] * a.d);
}

void kxyz_11x(const AxisCoef& ax, const AxisCoef& ay, const AxisCoef& az, dvec& kre, dvec& kim) {
  const int NX = ax.nm, NY = ay.nm, NZ = az.nm, NZ2 = NZ / 2 + 1;
  const double pi = std::acos(-1.0);
  dvec kx2, trx, ky2, tyy;
  waves_slip(ax, kx2, trx);
  waves_slip(ay, ky2, tyy);
  kre.assign((size_t)NX * NY * NZ2, 0.0);
  kim.assign(kre.size(), 0.0);
  if (az.periodic) {
    dvec kz2, trz;
    waves_tables(az, kz2, trz);
    for (int k = 0; k < NZ2; ++k)
      for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i) {
          const double txz = tyy[j] * trz[k], tyz = trx[i] * trz[k], txy = trx[i] * tyy[j];
          const double xt2 = kx2[i] * (txz * txz), yt2 = ky2[j] * (tyz * tyz), zt2 = kz2[k] * (txy * txy);
          const size_t q = (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k);
          kre[q] = xt2 + yt2 + zt2;
          kim[q] = kre[q];
        }
    return;
  }
  for (int k = 1; k <= NZ2; ++k) {
    const double w = pi * (double)(k - 1) / (double)NZ;
    const double w1 = pi * (double)(NZ - k + 1) / (double)NZ;
    double wp = az.aci6 * 2.0 * az.d * std::sin(w * 0.5) + (az.bci6 * 2.0 * az.d) * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * az.alcai6 * std::cos(w));
    double w1p = az.aci6 * 2.0 * az.d * std::sin(w1 * 0.5) + (az.bci6 * 2.0 * az.d) * std::sin(3.0 * 0.5 * w1);
    w1p = w1p / (1.0 + 2.0 * az.alcai6 * std::cos(w1));
    const double kzr = (double)NZ * wp / az.len, kzi = (double)NZ * w1p / az.len;
    const double zk2r = kzr * kzr, zk2i = kzi * kzi;
    const double rlezs = ((double)NZ * w / az.len) * az.d, iyezs = ((double)NZ * w1 / az.len) * az.d;
    const double ztr = 2.0 * (az.bici6 * std::cos(rlezs * 1.5) + az.cici6s * std::cos(rlezs * 2.5) +
                              az.dici6 * std::cos(rlezs * 3.5));
    const double zti = 2.0 * (az.bici6 * std::cos(iyezs * 1.5) + az.cici6s * std::cos(iyezs * 2.5) +
                              az.dici6 * std::cos(iyezs * 3.5));
    const double zt1r = 2.0 * az.aici6 * std::cos(rlezs * 0.5), zt1i = 2.0 * az.aici6 * std::cos(iyezs * 0.5);
    const double z1r = 1.0 + 2.0 * az.ailcai6 * std::cos(rlezs), z1i = 1.0 + 2.0 * az.ailcai6 * std::cos(iyezs);
    const double t1r = (zt1r + ztr) / z1r, t1i = (zt1i + zti) / z1i;
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i) {
        const double t2 = tyy[j], t3 = trx[i];
        const double t4r = t2 * t2 * (t1r * t1r), t4i = t2 * t2 * (t1i * t1i);
        const double t5r = t3 * t3 * (t1r * t1r), t5i = t3 * t3 * (t1i * t1i);
        const double t6 = (t3 * t2) * (t3 * t2);
        const size_t q = (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * (k - 1));
        kre[q] = t4r * kx2[i] + t5r * ky2[j] + t6 * zk2r;
        kim[q] = t4i * kx2[i] + t5i * ky2[j] + t6 * zk2i;
      }
  }
}

// A periodic plan whose Thomas factors (forward t_i -= s_i t_{i-1}, backward
// t_i = (t_i - f_i t_{i+1}) w_i) factor the corner-modified circulant that the
// periodic branches pair with the Sherman-Morrison correction: off-diagonals
// alpha, diagonal 2, 1, ..., 1, 1 + alpha^2.  Its solve is then A^-1 b with A
// = I + alpha (S + S^-1) circulant.  Coefficient sets built for other
// closures (e.g. the "p" sets of the staggered derivative on a periodic axis)
// are not.
bool plan_is_circulant(const OpPlan* p) {
  if (!p->periodic || p->nin != p->nout) return false;
  const double al = p->alpha;
  if (!(4.0 * al * al < 1.0)) return false;
  const int n = p->nout;
  const double tol = 1e-10;
  for (int i = 0; i < n; ++i) {
    const double diag = 1.0 / p->w[i] + (i > 0 ? p->s[i] * p->f[i - 1] : 0.0);
    const double want = (i == 0) ? 2.0 : (i == n - 1 ? 1.0 + al * al : 1.0);
    if (std::fabs(diag - want) > tol * want) return false;
    if (i < n - 1 && std::fabs(p->f[i] - al) > tol * std::fabs(al) + 1e-300) return false;
    if (i > 0 && std::fabs(p->s[i] / p->w[i - 1] - al) > tol * std::fabs(al) + 1e-300) return false;
  }
  return true;
}

}  // namespace x3d
