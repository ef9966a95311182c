// Parity oracle for the incompact3d_gb300 hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is a plain C++ restatement of the
// reference's FP64 CPU arithmetic for the per-timestep path.  It is linked by
// the tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and
// never by the product library.  Every routine cites the reference routine
// (path within the Incompact3d project, file:line) whose arithmetic it follows.
// Operation order inside each expression follows the Fortran source so that the
// oracle reproduces the reference to within a few ulp; build it with
// -ffp-contract=off so that no FMA contraction changes the rounding.
//
// Array layout: Fortran order (nx,ny,nz), x fastest, i.e. element (i,j,k)
// (0-based) at i + nx*(j + ny*k).
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::vector<double> vec;
typedef std::complex<double> cplx;

namespace {

const double PI = std::acos(-1.0);
const double TWOPI = 2.0 * std::acos(-1.0);

// ---------------------------------------------------------------------------
// Coefficient setup
// ---------------------------------------------------------------------------

// Thomas LU factorisation: src/schemes.f90:413-439 (prepare).
void prepare(const vec& b, const vec& c, const vec& f, vec& s, vec& w, int n) {
  for (int i = 0; i < n; ++i) w[i] = c[i];
  for (int i = 1; i < n; ++i) {
    s[i] = b[i - 1] / w[i - 1];
    w[i] = w[i] - f[i - 1] * s[i];
  }
  for (int i = 0; i < n; ++i) w[i] = 1.0 / w[i];
}

struct Axis {
  int n = 0, nm = 0, ncl1 = 0, ncln = 0;
  bool periodic = true;
  double len = 0, d = 0, d2 = 0;
  // first derivative (module derivX/Y/Z scalars, src/module_param.f90:559-617)
  double alfa1, af1, bf1, cf1, df1, alfa2, af2, alfan, afn, bfn, cfn, dfn, alfam, afm, alfai, afi, bfi;
  vec ff, fs, fw, ffp, fsp, fwp;
  // second derivative
  double alsa1, as1, bs1, cs1, ds1, alsa2, as2, alsan, asn, bsn, csn, dsn, alsam, asm_, alsa3, as3, bs3,
      alsat, ast, bst, alsa4, as4, bs4, cs4, alsatt, astt, bstt, cstt, alsai, asi, bsi, csi, dsi;
  vec sf, ss, sw, sfp, ssp, swp;
  // staggered derivative / interpolation
  double alcai6, aci6, bci6, ailcai6, aici6, bici6, cicoef6, dici6;
  vec cf6, cc6, cb6, cfp6, ciwp6, csp6, cwp6, cs6, cw6, cif6, cic6, cis6, cib6, cifp6, cisp6, ciw6;  // nm
  vec cfi6, cci6, cbi6, cfip6, csip6, cwip6, csi6, cwi6, cifi6, cici6, cibi6, cifip6, cisip6, ciwip6, cisi6,
      ciwi6;  // n
  // filter (module parfiX/Y/Z)
  double fial1, fia1, fib1, fic1, fid1, fial2, fia2, fib2, fic2, fid2, fial3, fia3, fib3, fic3, fid3, fie3, fif3,
      fialn, fian, fibn, ficn, fidn, fialm, fiam, fibm, ficm, fidm, fialp, fiap, fibp, ficp, fidp, fiep, fifp,
      fiali, fiai, fibi, fici, fidi;
  vec fiff, fifs, fifw, fiffp, fifsp, fifwp;
};

struct Opts {
  int ifirstder = 4, isecondder = 4, ipinter = 3;
  double nu0nu = 4.0, cnu = 0.44, filter_alpha = 0.49;
};

// src/schemes.f90:443-599 (first_derivative)
void first_derivative(Axis& a, const Opts& o) {
  const int n = a.n;
  const double d = a.d;
  a.ff.assign(n, 0); a.fs.assign(n, 0); a.fw.assign(n, 0);
  a.ffp.assign(n, 0); a.fsp.assign(n, 0); a.fwp.assign(n, 0);
  vec fb(n, 0.0), fc(n, 0.0);
  if (o.ifirstder == 1) {
    a.alfai = 0.0; a.afi = 1.0 / (2.0 * d); a.bfi = 0.0;
  } else {
    a.alfai = 1.0 / 3.0; a.afi = (7.0 / 9.0) / d; a.bfi = (1.0 / 36.0) / d;
  }
  if (o.ifirstder == 1) {
    a.alfa1 = a.af1 = a.bf1 = a.cf1 = a.df1 = a.alfa2 = a.af2 = 0;
    a.alfam = a.afm = a.alfan = a.afn = a.bfn = a.cfn = a.dfn = 0;
  } else {
    a.alfa1 = 2.0; a.af1 = -(5.0 / 2.0) / d; a.bf1 = 2.0 / d; a.cf1 = 0.5 / d; a.df1 = 0.0;
    a.alfa2 = 1.0 / 4.0; a.af2 = (3.0 / 4.0) / d;
    a.alfan = 2.0; a.afn = -(5.0 / 2.0) / d; a.bfn = 2.0 / d; a.cfn = 0.5 / d; a.dfn = 0.0;
    a.alfam = 1.0 / 4.0; a.afm = (3.0 / 4.0) / d;
  }
  if (n == 1) return;
  vec& ff = a.ff;
  const double al = a.alfai;
  if (a.ncl1 == 0) { ff[0] = al; ff[1] = al; fc[0] = 2.0; fc[1] = 1.0; fb[0] = al; fb[1] = al; }
  else if (a.ncl1 == 1) { ff[0] = al + al; ff[1] = al; fc[0] = 1.0; fc[1] = 1.0; fb[0] = al; fb[1] = al; }
  else { ff[0] = a.alfa1; ff[1] = a.alfa2; fc[0] = 1.0; fc[1] = 1.0; fb[0] = a.alfa2; fb[1] = al; }
  if (a.ncln == 0) {
    ff[n - 3] = al; ff[n - 2] = al; ff[n - 1] = 0; fc[n - 3] = 1; fc[n - 2] = 1; fc[n - 1] = 1.0 + al * al;
    fb[n - 3] = al; fb[n - 2] = al; fb[n - 1] = 0;
  } else if (a.ncln == 1) {
    ff[n - 3] = al; ff[n - 2] = al; ff[n - 1] = 0; fc[n - 3] = 1; fc[n - 2] = 1; fc[n - 1] = 1;
    fb[n - 3] = al; fb[n - 2] = al + al; fb[n - 1] = 0;
  } else {
    ff[n - 3] = al; ff[n - 2] = a.alfam; ff[n - 1] = 0; fc[n - 3] = 1; fc[n - 2] = 1; fc[n - 1] = 1;
    fb[n - 3] = a.alfam; fb[n - 2] = a.alfan; fb[n - 1] = 0;
  }
  for (int i = 2; i < n - 3; ++i) { ff[i] = al; fc[i] = 1.0; fb[i] = al; }
  for (int i = 0; i < n; ++i) a.ffp[i] = ff[i];
  prepare(fb, fc, a.ff, a.fs, a.fw, n);
  if (a.ncl1 == 1) a.ffp[0] = 0.0;
  if (a.ncln == 1) fb[n - 2] = 0.0;
  prepare(fb, fc, a.ffp, a.fsp, a.fwp, n);
}

// src/schemes.f90:602-856 (second_derivative)
void second_derivative(Axis& a, const Opts& o) {
  const int n = a.n;
  const double d2 = a.d2;
  a.sf.assign(n, 0); a.ss.assign(n, 0); a.sw.assign(n, 0);
  a.sfp.assign(n, 0); a.ssp.assign(n, 0); a.swp.assign(n, 0);
  vec sb(n, 0.0), sc(n, 0.0);
  if (o.isecondder == 1) {
    a.alsai = 0; a.asi = 1.0 / d2; a.bsi = 0; a.csi = 0; a.dsi = 0;
  } else if (o.isecondder == 4) {
    a.alsai = 2.0 / 11.0; a.asi = (12.0 / 11.0) / d2; a.bsi = (3.0 / 44.0) / d2; a.csi = 0; a.dsi = 0;
  } else if (o.isecondder == 5) {
    const double dpis3 = 2.0 * PI / 3.0;
    const double kppkc = PI * PI * (1.0 + o.nu0nu);
    const double kppkm = dpis3 * dpis3 * (1.0 + o.cnu * o.nu0nu);
    const double xnpi2 = kppkc, xmpi2 = kppkm;
    const double den = 405.0 * xnpi2 - 640.0 * xmpi2 + 144.0;
    a.alsai = 0.5 - (320.0 * xmpi2 - 1296.0) / den;
    a.asi = -(4329.0 * xnpi2 / 8.0 - 32.0 * xmpi2 - 140.0 * xnpi2 * xmpi2 + 286.0) / den / d2;
    a.bsi = (2115.0 * xnpi2 - 1792.0 * xmpi2 - 280.0 * xnpi2 * xmpi2 + 1328.0) / den / (4.0 * d2);
    a.csi = -(7695.0 * xnpi2 / 8.0 + 288.0 * xmpi2 - 180.0 * xnpi2 * xmpi2 - 2574.0) / den / (9.0 * d2);
    a.dsi = (198.0 * xnpi2 + 128.0 * xmpi2 - 40.0 * xnpi2 * xmpi2 - 736.0) / den / (16.0 * d2);
  }
  a.alsa1 = 11.0; a.as1 = 13.0 / d2; a.bs1 = -27.0 / d2; a.cs1 = 15.0 / d2; a.ds1 = -1.0 / d2;
  if (o.isecondder == 1) { a.alsa2 = 0; a.as2 = 1.0 / d2; } else { a.alsa2 = 0.1; a.as2 = (6.0 / 5.0) / d2; }
  a.alsa3 = 2.0 / 11.0; a.as3 = (12.0 / 11.0) / d2; a.bs3 = (3.0 / 44.0) / d2;
  a.alsa4 = 2.0 / 11.0; a.as4 = (12.0 / 11.0) / d2; a.bs4 = (3.0 / 44.0) / d2; a.cs4 = 0;
  a.alsan = 11.0; a.asn = 13.0 / d2; a.bsn = -27.0 / d2; a.csn = 15.0 / d2; a.dsn = -1.0 / d2;
  if (o.isecondder == 1) { a.alsam = 0; a.asm_ = 1.0 / d2; } else { a.alsam = 0.1; a.asm_ = (6.0 / 5.0) / d2; }
  a.alsat = 2.0 / 11.0; a.ast = (12.0 / 11.0) / d2; a.bst = (3.0 / 44.0) / d2;
  a.alsatt = 2.0 / 11.0; a.astt = (12.0 / 11.0) / d2; a.bstt = (3.0 / 44.0) / d2; a.cstt = 0;
  if (n == 1) return;
  vec& sf = a.sf;
  const double al = a.alsai;
  if (a.ncl1 == 0) {
    for (int i = 0; i < 4; ++i) { sf[i] = al; sc[i] = 1.0; sb[i] = al; }
    sc[0] = 2.0;
  } else if (a.ncl1 == 1) {
    for (int i = 0; i < 4; ++i) { sf[i] = al; sc[i] = 1.0; sb[i] = al; }
    sf[0] = al + al;
  } else {
    sf[0] = a.alsa1; sf[1] = a.alsa2; sf[2] = a.alsa3; sf[3] = a.alsa4;
    sc[0] = sc[1] = sc[2] = sc[3] = 1.0;
    sb[0] = a.alsa2; sb[1] = a.alsa3; sb[2] = a.alsa4; sb[3] = al;
  }
  if (a.ncln == 0) {
    for (int i = n - 5; i < n - 1; ++i) { sf[i] = al; sc[i] = 1.0; sb[i] = al; }
    sf[n - 1] = 0; sc[n - 1] = 1.0 + al * al; sb[n - 1] = 0;
  } else if (a.ncln == 1) {
    for (int i = n - 5; i < n - 1; ++i) { sf[i] = al; sc[i] = 1.0; sb[i] = al; }
    sf[n - 1] = 0; sc[n - 1] = 1.0; sb[n - 2] = al + al; sb[n - 1] = 0;
  } else {
    sf[n - 5] = al; sf[n - 4] = a.alsatt; sf[n - 3] = a.alsat; sf[n - 2] = a.alsam; sf[n - 1] = 0;
    for (int i = n - 5; i < n; ++i) sc[i] = 1.0;
    sb[n - 5] = a.alsatt; sb[n - 4] = a.alsat; sb[n - 3] = a.alsam; sb[n - 2] = a.alsan; sb[n - 1] = 0;
  }
  for (int i = 4; i < n - 5; ++i) { sf[i] = al; sc[i] = 1.0; sb[i] = al; }
  for (int i = 0; i < n; ++i) a.sfp[i] = sf[i];
  if (a.ncl1 == 1) sf[0] = 0.0;
  prepare(sb, sc, a.sf, a.ss, a.sw, n);
  prepare(sb, sc, a.sfp, a.ssp, a.swp, n);
  if (a.ncln == 1) {
    sb[n - 2] = 0.0;
    prepare(sb, sc, a.sf, a.ss, a.sw, n);
  }
}

// src/schemes.f90:860-1066 (interpolation)
void interpolation(Axis& a, const Opts& o) {
  const int nx = a.n, nxm = a.nm;
  const double dx = a.d;
  if (o.ifirstder == 1) {
    a.alcai6 = 0; a.aci6 = 1.0 / dx; a.bci6 = 0;
  } else {
    a.alcai6 = 9.0 / 62.0; a.aci6 = (63.0 / 62.0) / dx; a.bci6 = (17.0 / 62.0) / 3.0 / dx;
  }
  if (o.ifirstder == 1) {
    a.ailcai6 = 0; a.aici6 = 0.5; a.bici6 = a.cicoef6 = a.dici6 = 0;
  } else if (o.ipinter == 1) {
    a.ailcai6 = 3.0 / 10.0; a.aici6 = 3.0 / 4.0; a.bici6 = 1.0 / (2.0 * 10.0); a.cicoef6 = 0; a.dici6 = 0;
  } else if (o.ipinter == 2) {
    a.ailcai6 = 0.461658;
    a.dici6 = 0.00293016;
    a.aici6 = 1.0 / 64.0 * (75.0 + 70.0 * a.ailcai6 - 320.0 * a.dici6);
    a.bici6 = 1.0 / 128.0 * (126.0 * a.ailcai6 - 25.0 + 1152.0 * a.dici6);
    a.cicoef6 = 1.0 / 128.0 * (-10.0 * a.ailcai6 + 3.0 - 640.0 * a.dici6);
    a.aici6 = a.aici6 / 2.0; a.bici6 = a.bici6 / 2.0; a.cicoef6 = a.cicoef6 / 2.0; a.dici6 = a.dici6 / 2.0;
  } else {
    a.ailcai6 = 0.49;
    a.aici6 = 1.0 / 128.0 * (75.0 + 70.0 * a.ailcai6);
    a.bici6 = 1.0 / 256.0 * (126.0 * a.ailcai6 - 25.0);
    a.cicoef6 = 1.0 / 256.0 * (-10.0 * a.ailcai6 + 3.0);
    a.dici6 = 0;
  }
  vec* m6[] = {&a.cf6, &a.cc6, &a.cb6, &a.cfp6, &a.ciwp6, &a.csp6, &a.cwp6, &a.cs6,
               &a.cw6, &a.cif6, &a.cic6, &a.cis6, &a.cib6, &a.cifp6, &a.cisp6, &a.ciw6};
  for (vec* v : m6) v->assign(nxm, 0.0);
  vec* i6[] = {&a.cfi6, &a.cci6, &a.cbi6, &a.cfip6, &a.csip6, &a.cwip6, &a.csi6, &a.cwi6,
               &a.cifi6, &a.cici6, &a.cibi6, &a.cifip6, &a.cisip6, &a.ciwip6, &a.cisi6, &a.ciwi6};
  for (vec* v : i6) v->assign(nx, 0.0);
  if (nx == 1) return;
  const double al = a.alcai6, ail = a.ailcai6;
  vec &cfx6 = a.cf6, &ccx6 = a.cc6, &cbx6 = a.cb6;
  cfx6[0] = al; cfx6[1] = al; cfx6[nxm - 3] = al; cfx6[nxm - 2] = al; cfx6[nxm - 1] = 0;
  if (a.ncl1 == 0) ccx6[0] = 2.0; else ccx6[0] = 1.0 + al;
  ccx6[1] = 1; ccx6[nxm - 3] = 1; ccx6[nxm - 2] = 1;
  if (a.ncln == 0) ccx6[nxm - 1] = 1.0 + al * al; else ccx6[nxm - 1] = 1.0 + al;
  cbx6[0] = al; cbx6[1] = al; cbx6[nxm - 3] = al; cbx6[nxm - 2] = al; cbx6[nxm - 1] = 0;
  for (int i = 2; i < nxm - 3; ++i) { cfx6[i] = al; ccx6[i] = 1; cbx6[i] = al; }
  vec &cfi6 = a.cfi6, &cci6 = a.cci6, &cbi6 = a.cbi6;
  cfi6[0] = al + al; cfi6[1] = al; cfi6[nx - 3] = al; cfi6[nx - 2] = al; cfi6[nx - 1] = 0;
  cci6[0] = 1; cci6[1] = 1; cci6[nx - 3] = 1; cci6[nx - 2] = 1; cci6[nx - 1] = 1;
  cbi6[0] = al; cbi6[1] = al; cbi6[nx - 3] = al; cbi6[nx - 2] = al + al; cbi6[nx - 1] = 0;
  for (int i = 2; i < nx - 3; ++i) { cfi6[i] = al; cci6[i] = 1; cbi6[i] = al; }
  vec &cifx6 = a.cif6, &cicx6 = a.cic6, &cibx6 = a.cib6;
  cifx6[0] = ail; cifx6[1] = ail; cifx6[nxm - 3] = ail; cifx6[nxm - 2] = ail; cifx6[nxm - 1] = 0;
  if (a.ncl1 == 0) cicx6[0] = 2.0; else cicx6[0] = 1.0 + ail;
  cicx6[1] = 1; cicx6[nxm - 3] = 1; cicx6[nxm - 2] = 1;
  if (a.ncln == 0) cicx6[nxm - 1] = 1.0 + ail * ail; else cicx6[nxm - 1] = 1.0 + ail;
  cibx6[0] = ail; cibx6[1] = ail; cibx6[nxm - 3] = ail; cibx6[nxm - 2] = ail; cibx6[nxm - 1] = 0;
  for (int i = 2; i < nxm - 3; ++i) { cifx6[i] = ail; cicx6[i] = 1; cibx6[i] = ail; }
  vec &cifi6 = a.cifi6, &cici6 = a.cici6, &cibi6 = a.cibi6;
  cifi6[0] = ail + ail; cifi6[1] = ail; cifi6[nx - 3] = ail; cifi6[nx - 2] = ail; cifi6[nx - 1] = 0;
  cici6[0] = 1; cici6[1] = 1; cici6[nx - 3] = 1; cici6[nx - 2] = 1; cici6[nx - 1] = 1;
  cibi6[0] = ail; cibi6[1] = ail; cibi6[nx - 3] = ail; cibi6[nx - 2] = ail + ail; cibi6[nx - 1] = 0;
  for (int i = 2; i < nx - 3; ++i) { cifi6[i] = ail; cici6[i] = 1; cibi6[i] = ail; }
  for (int i = 0; i < nxm; ++i) { a.cfp6[i] = cfx6[i]; a.cifp6[i] = cifx6[i]; }
  for (int i = 0; i < nx; ++i) { a.cifip6[i] = cifi6[i]; a.cfip6[i] = cfi6[i]; }
  a.cfp6[0] = 0; a.cfip6[0] = 0;
  prepare(cbx6, ccx6, cfx6, a.cs6, a.cw6, nxm);
  prepare(cbx6, ccx6, a.cfp6, a.csp6, a.cwp6, nxm);
  prepare(cibx6, cicx6, cifx6, a.cis6, a.ciw6, nxm);
  prepare(cibx6, cicx6, a.cifp6, a.cisp6, a.ciwp6, nxm);
  prepare(cbi6, cci6, cfi6, a.csi6, a.cwi6, nx);
  prepare(cbi6, cci6, a.cfip6, a.csip6, a.cwip6, nx);
  prepare(cibi6, cici6, cifi6, a.cisi6, a.ciwi6, nx);
  prepare(cibi6, cici6, a.cifip6, a.cisip6, a.ciwip6, nx);
  if (a.ncln == 1 || a.ncln == 2) {
    cbx6[nxm - 2] = 0; cibx6[nxm - 1] = 0; cbi6[nx - 2] = 0; cibi6[nx - 1] = 0;
    prepare(cbx6, ccx6, a.cfp6, a.csp6, a.cwp6, nxm);
    prepare(cibx6, cicx6, a.cifp6, a.cisp6, a.ciwp6, nxm);
    prepare(cbi6, cci6, a.cfip6, a.csip6, a.cwip6, nx);
    prepare(cibi6, cici6, a.cifip6, a.cisip6, a.ciwip6, nx);
  }
}

// src/filters.f90:62-219 (set_filter_coefficients)
void filter_coefficients(Axis& a, double af) {
  const int n = a.n;
  a.fiali = af;
  a.fiai = (11.0 + 10.0 * af) / 16.0;
  a.fibi = 0.5 * (15.0 + 34.0 * af) / 32.0;
  a.fici = 0.5 * (-3.0 + 6.0 * af) / 16.0;
  a.fidi = 0.5 * (1.0 - 2.0 * af) / 32.0;
  a.fial1 = 0; a.fia1 = 1; a.fib1 = 0; a.fic1 = 0; a.fid1 = 0;
  a.fial2 = af; a.fia2 = 1.0 / 8.0 + 3.0 / 4.0 * af; a.fib2 = 5.0 / 8.0 + 3.0 / 4.0 * af;
  a.fic2 = 3.0 / 8.0 + af / 4.0; a.fid2 = -1.0 / 8.0 + af / 4.0;
  a.fial3 = af; a.fia3 = -1.0 / 32.0 + af / 16.0; a.fib3 = 5.0 / 32.0 + 11.0 / 16.0 * af;
  a.fic3 = 11.0 / 16.0 + 5.0 * af / 8.0; a.fid3 = 5.0 / 16.0 + 3.0 * af / 8.0;
  a.fie3 = -5.0 / 32.0 + 5.0 * af / 16.0; a.fif3 = 1.0 / 32.0 - af / 16.0;
  a.fialn = 0; a.fian = 1; a.fibn = 0; a.ficn = 0; a.fidn = 0;
  a.fialm = af; a.fiam = 1.0 / 8.0 + 3.0 / 4.0 * af; a.fibm = 5.0 / 8.0 + 3.0 / 4.0 * af;
  a.ficm = 3.0 / 8.0 + af / 4.0; a.fidm = -1.0 / 8.0 + af / 4.0;
  a.fialp = af; a.fiap = -1.0 / 32.0 + af / 16.0; a.fibp = 5.0 / 32.0 + 11.0 / 16.0 * af;
  a.ficp = 11.0 / 16.0 + 5.0 * af / 8.0; a.fidp = 5.0 / 16.0 + 3.0 * af / 8.0;
  a.fiep = -5.0 / 32.0 + 5.0 * af / 16.0; a.fifp = 1.0 / 32.0 - af / 16.0;
  a.fiff.assign(n, 0); a.fifs.assign(n, 0); a.fifw.assign(n, 0);
  a.fiffp.assign(n, 0); a.fifsp.assign(n, 0); a.fifwp.assign(n, 0);
  vec fb(n, 0.0), fc(n, 0.0);
  vec& ff = a.fiff;
  const double al = a.fiali;
  if (a.ncl1 == 0) { ff[0] = al; ff[1] = al; fc[0] = 2; fc[1] = 1; fb[0] = al; fb[1] = al; }
  else if (a.ncl1 == 1) { ff[0] = al + al; ff[1] = al; fc[0] = 1; fc[1] = 1; fb[0] = al; fb[1] = al; }
  else { ff[0] = a.fial1; ff[1] = a.fial2; fc[0] = 1; fc[1] = 1; fb[0] = a.fial2; fb[1] = al; }
  if (a.ncln == 0) {
    ff[n - 3] = al; ff[n - 2] = al; ff[n - 1] = 0; fc[n - 3] = 1; fc[n - 2] = 1; fc[n - 1] = 1.0 + al * al;
    fb[n - 3] = al; fb[n - 2] = al; fb[n - 1] = 0;
  } else if (a.ncln == 1) {
    ff[n - 3] = al; ff[n - 2] = al; ff[n - 1] = 0; fc[n - 3] = 1; fc[n - 2] = 1; fc[n - 1] = 1;
    fb[n - 3] = al; fb[n - 2] = al + al; fb[n - 1] = 0;
  } else {
    ff[n - 3] = al; ff[n - 2] = a.fialm; ff[n - 1] = 0; fc[n - 3] = 1; fc[n - 2] = 1; fc[n - 1] = 1;
    fb[n - 3] = a.fialm; fb[n - 2] = a.fialn; fb[n - 1] = 0;
  }
  for (int i = 2; i < n - 3; ++i) { ff[i] = al; fc[i] = 1; fb[i] = al; }
  for (int i = 0; i < n; ++i) a.fiffp[i] = ff[i];
  prepare(fb, fc, a.fiffp, a.fifsp, a.fifwp, n);
  if (a.ncl1 == 1) ff[0] = 0;
  if (a.ncln == 1) fb[n - 2] = 0;
  prepare(fb, fc, a.fiff, a.fifs, a.fifw, n);
}

// ---------------------------------------------------------------------------
// Line operators.  Each one restates, for a single line, the arithmetic that
// the reference applies to every x-, y- or z-line (the y and z versions of each
// routine repeat the x version's per-line arithmetic with their own coefficient
// module).  U(i) / T(i) are 1-based accessors so the formulas read like the
// Fortran.
// ---------------------------------------------------------------------------

enum { OP_DER1 = 0, OP_DER2 = 1, OP_FIL = 2, OP_DVP = 3, OP_IVP = 4, OP_DPV = 5, OP_IPV = 6 };

#define U(i) u[(i) - 1]
#define T(i) t[(i) - 1]
#define R(i) r[(i) - 1]

// Forward/backward Thomas sweeps shared by every routine:
// t(i) -= t(i-1)*s(i); t(n) *= w(n); t(i) = (t(i) - f(i)*t(i+1))*w(i).
void thomas(double* t, int n, const vec& f, const vec& s, const vec& w) {
  for (int i = 2; i <= n; ++i) T(i) = T(i) - T(i - 1) * s[i - 1];
  T(n) = T(n) * w[n - 1];
  for (int i = n - 1; i >= 1; --i) T(i) = (T(i) - f[i - 1] * T(i + 1)) * w[i - 1];
}

// Periodic Sherman-Morrison correction, e.g. src/derive.f90:27-56 (derx_00):
// r = (-1, 0, ..., 0, alpha) swept with the same factors, then
// s = (t1 - alpha tn)/(1 + r1 - alpha rn); t -= s r.
void sherman_morrison(double* t, int n, double alpha, const vec& f, const vec& s, const vec& w) {
  vec rr(n, 0.0);
  double* r = rr.data();
  R(1) = -1.0;
  R(n) = alpha;
  for (int i = 2; i <= n; ++i) R(i) = R(i) - R(i - 1) * s[i - 1];
  R(n) = R(n) * w[n - 1];
  for (int i = n - 1; i >= 1; --i) R(i) = (R(i) - f[i - 1] * R(i + 1)) * w[i - 1];
  const double sx = (T(1) - alpha * T(n)) / (1.0 + R(1) - alpha * R(n));
  for (int i = 1; i <= n; ++i) T(i) = T(i) - sx * R(i);
}

// First derivative RHS: src/derive.f90:7-321 (derx_00/11/12/21/22).
void der1_line(const Axis& a, int npaire, const double* u, double* t) {
  const int nx = a.n;
  const double afi = a.afi, bfi = a.bfi;
  const int c1 = a.ncl1, cn = a.ncln;
  if (c1 == 0 && cn == 0) {
    T(1) = afi * (U(2) - U(nx)) + bfi * (U(3) - U(nx - 1));
    T(2) = afi * (U(3) - U(1)) + bfi * (U(4) - U(nx));
    for (int i = 3; i <= nx - 2; ++i) T(i) = afi * (U(i + 1) - U(i - 1)) + bfi * (U(i + 2) - U(i - 2));
    T(nx - 1) = afi * (U(nx) - U(nx - 2)) + bfi * (U(1) - U(nx - 3));
    T(nx) = afi * (U(1) - U(nx - 1)) + bfi * (U(2) - U(nx - 2));
    return;
  }
  // left end
  if (c1 == 1) {
    if (npaire == 1) {
      T(1) = 0.0;
      T(2) = afi * (U(3) - U(1)) + bfi * (U(4) - U(2));
    } else {
      T(1) = afi * (U(2) + U(2)) + bfi * (U(3) + U(3));
      T(2) = afi * (U(3) - U(1)) + bfi * (U(4) + U(2));
    }
  } else {  // Dirichlet
    T(1) = a.af1 * U(1) + a.bf1 * U(2) + a.cf1 * U(3);
    T(2) = a.af2 * (U(3) - U(1));
  }
  for (int i = 3; i <= nx - 2; ++i) T(i) = afi * (U(i + 1) - U(i - 1)) + bfi * (U(i + 2) - U(i - 2));
  // right end
  if (cn == 1) {
    if (npaire == 1) {
      T(nx - 1) = afi * (U(nx) - U(nx - 2)) + bfi * (U(nx - 1) - U(nx - 3));
      T(nx) = 0.0;
    } else {
      T(nx - 1) = afi * (U(nx) - U(nx - 2)) + bfi * ((-U(nx - 1)) - U(nx - 3));
      T(nx) = afi * ((-U(nx - 1)) - U(nx - 1)) + bfi * ((-U(nx - 2)) - U(nx - 2));
    }
  } else {
    T(nx - 1) = a.afm * (U(nx) - U(nx - 2));
    T(nx) = (-a.afn * U(nx)) - a.bfn * U(nx - 1) - a.cfn * U(nx - 2);
  }
}

inline double d2term(const double* u, int ip, int i, int im) { return U(ip) - U(i) - U(i) + U(im); }

// Second derivative RHS: src/derive.f90:1354-2048 (derxx_00/11/12/21/22).
void der2_line(const Axis& a, int npaire, const double* u, double* t) {
  const int nx = a.n;
  const double as = a.asi, bs = a.bsi, cs = a.csi, ds = a.dsi;
  const int c1 = a.ncl1, cn = a.ncln;
  auto wrap = [nx](int i) { return ((i - 1) % nx + nx) % nx + 1; };
  auto interior = [&](int i) {
    return as * (U(i + 1) - U(i) - U(i) + U(i - 1)) + bs * (U(i + 2) - U(i) - U(i) + U(i - 2)) +
           cs * (U(i + 3) - U(i) - U(i) + U(i - 3)) + ds * (U(i + 4) - U(i) - U(i) + U(i - 4));
  };
  if (c1 == 0 && cn == 0) {
    for (int i = 1; i <= nx; ++i) {
      if (i >= 5 && i <= nx - 4) { T(i) = interior(i); continue; }
      T(i) = as * (U(wrap(i + 1)) - U(i) - U(i) + U(wrap(i - 1))) +
             bs * (U(wrap(i + 2)) - U(i) - U(i) + U(wrap(i - 2))) +
             cs * (U(wrap(i + 3)) - U(i) - U(i) + U(wrap(i - 3))) +
             ds * (U(wrap(i + 4)) - U(i) - U(i) + U(wrap(i - 4)));
    }
    return;
  }
  // left end
  if (c1 == 1) {
    if (npaire == 1) {
      T(1) = as * (U(2) - U(1) - U(1) + U(2)) + bs * (U(3) - U(1) - U(1) + U(3)) +
             cs * (U(4) - U(1) - U(1) + U(4)) + ds * (U(5) - U(1) - U(1) + U(5));
      T(2) = as * (U(3) - U(2) - U(2) + U(1)) + bs * (U(4) - U(2) - U(2) + U(2)) +
             cs * (U(5) - U(2) - U(2) + U(3)) + ds * (U(6) - U(2) - U(2) + U(4));
      T(3) = as * (U(4) - U(3) - U(3) + U(2)) + bs * (U(5) - U(3) - U(3) + U(1)) +
             cs * (U(6) - U(3) - U(3) + U(2)) + ds * (U(7) - U(3) - U(3) + U(3));
      T(4) = as * (U(5) - U(4) - U(4) + U(3)) + bs * (U(6) - U(4) - U(4) + U(2)) +
             cs * (U(7) - U(4) - U(4) + U(1)) + ds * (U(8) - U(4) - U(4) + U(2));
    } else {
      T(1) = 0.0;
      T(2) = as * (U(3) - U(2) - U(2) + U(1)) + bs * (U(4) - U(2) - U(2) - U(2)) +
             cs * (U(5) - U(2) - U(2) - U(3)) + ds * (U(6) - U(2) - U(2) - U(4));
      T(3) = as * (U(4) - U(3) - U(3) + U(2)) + bs * (U(5) - U(3) - U(3) + U(1)) +
             cs * (U(6) - U(3) - U(3) - U(2)) + ds * (U(7) - U(3) - U(3) - U(3));
      T(4) = as * (U(5) - U(4) - U(4) + U(3)) + bs * (U(6) - U(4) - U(4) + U(2)) +
             cs * (U(7) - U(4) - U(4) - U(1)) + ds * (U(8) - U(4) - U(4) - U(2));
    }
  } else {  // Dirichlet (derxx_21/22 left rows)
    T(1) = a.as1 * U(1) + a.bs1 * U(2) + a.cs1 * U(3) + a.ds1 * U(4);
    T(2) = a.as2 * (U(3) - U(2) - U(2) + U(1));
    T(3) = a.as3 * (U(4) - U(3) - U(3) + U(2)) + a.bs3 * (U(5) - U(3) - U(3) + U(1));
    T(4) = a.as4 * (U(5) - U(4) - U(4) + U(3)) + a.bs4 * (U(6) - U(4) - U(4) + U(2)) +
           a.cs4 * (U(7) - U(4) - U(4) + U(1));
  }
  for (int i = 5; i <= nx - 4; ++i) T(i) = interior(i);
  // right end
  if (cn == 1) {
    if (npaire == 1) {
      T(nx - 3) = as * (U(nx - 2) - U(nx - 3) - U(nx - 3) + U(nx - 4)) +
                  bs * (U(nx - 1) - U(nx - 3) - U(nx - 3) + U(nx - 5)) +
                  cs * (U(nx) - U(nx - 3) - U(nx - 3) + U(nx - 6)) +
                  ds * (U(nx - 1) - U(nx - 3) - U(nx - 3) + U(nx - 7));
      T(nx - 2) = as * (U(nx - 1) - U(nx - 2) - U(nx - 2) + U(nx - 3)) +
                  bs * (U(nx) - U(nx - 2) - U(nx - 2) + U(nx - 4)) +
                  cs * (U(nx - 1) - U(nx - 2) - U(nx - 2) + U(nx - 5)) +
                  ds * (U(nx - 2) - U(nx - 2) - U(nx - 2) + U(nx - 6));
      T(nx - 1) = as * (U(nx) - U(nx - 1) - U(nx - 1) + U(nx - 2)) +
                  bs * (U(nx - 1) - U(nx - 1) - U(nx - 1) + U(nx - 3)) +
                  cs * (U(nx - 2) - U(nx - 1) - U(nx - 1) + U(nx - 4)) +
                  ds * (U(nx - 3) - U(nx - 1) - U(nx - 1) + U(nx - 5));
      T(nx) = as * (U(nx - 1) - U(nx) - U(nx) + U(nx - 1)) + bs * (U(nx - 2) - U(nx) - U(nx) + U(nx - 2)) +
              cs * (U(nx - 3) - U(nx) - U(nx) + U(nx - 3)) + ds * (U(nx - 4) - U(nx) - U(nx) + U(nx - 4));
    } else {
      T(nx - 3) = as * (U(nx - 2) - U(nx - 3) - U(nx - 3) + U(nx - 4)) +
                  bs * (U(nx - 1) - U(nx - 3) - U(nx - 3) + U(nx - 5)) +
                  cs * (-U(nx) - U(nx - 3) - U(nx - 3) + U(nx - 6)) +
                  ds * (-U(nx - 1) - U(nx - 3) - U(nx - 3) + U(nx - 7));
      T(nx - 2) = as * (U(nx - 1) - U(nx - 2) - U(nx - 2) + U(nx - 3)) +
                  bs * (U(nx) - U(nx - 2) - U(nx - 2) + U(nx - 4)) +
                  cs * (-U(nx - 1) - U(nx - 2) - U(nx - 2) + U(nx - 5)) +
                  ds * (-U(nx - 2) - U(nx - 2) - U(nx - 2) + U(nx - 6));
      T(nx - 1) = as * (U(nx) - U(nx - 1) - U(nx - 1) + U(nx - 2)) +
                  bs * (-U(nx - 1) - U(nx - 1) - U(nx - 1) + U(nx - 3)) +
                  cs * (-U(nx - 2) - U(nx - 1) - U(nx - 1) + U(nx - 4)) +
                  ds * (-U(nx - 3) - U(nx - 1) - U(nx - 1) + U(nx - 5));
      T(nx) = 0.0;
    }
  } else {  // Dirichlet (derxx_12/22 right rows)
    T(nx - 3) = a.astt * (U(nx - 2) - U(nx - 3) - U(nx - 3) + U(nx - 4)) +
                a.bstt * (U(nx - 1) - U(nx - 3) - U(nx - 3) + U(nx - 5)) +
                a.cstt * (U(nx) - U(nx - 3) - U(nx - 3) + U(nx - 6));
    T(nx - 2) = a.ast * (U(nx - 1) - U(nx - 2) - U(nx - 2) + U(nx - 3)) +
                a.bst * (U(nx) - U(nx - 2) - U(nx - 2) + U(nx - 4));
    T(nx - 1) = a.asm_ * (U(nx) - U(nx - 1) - U(nx - 1) + U(nx - 2));
    T(nx) = a.asn * U(nx) + a.bsn * U(nx - 1) + a.csn * U(nx - 2) + a.dsn * U(nx - 3);
  }
}

// Filter RHS: src/filters.f90:221-605 (filx_00/11/12/21/22).
void fil_line(const Axis& a, int npaire, const double* u, double* t) {
  const int nx = a.n;
  const double fa = a.fiai, fb = a.fibi, fc = a.fici, fd = a.fidi;
  const int c1 = a.ncl1, cn = a.ncln;
  auto wrap = [nx](int i) { return ((i - 1) % nx + nx) % nx + 1; };
  if (c1 == 0 && cn == 0) {
    for (int i = 1; i <= nx; ++i)
      T(i) = fa * U(i) + fb * (U(wrap(i + 1)) + U(wrap(i - 1))) + fc * (U(wrap(i + 2)) + U(wrap(i - 2))) +
             fd * (U(wrap(i + 3)) + U(wrap(i - 3)));
    return;
  }
  if (c1 == 1) {
    if (npaire == 1) {
      T(1) = fa * U(1) + fb * (U(2) + U(2)) + fc * (U(3) + U(3)) + fd * (U(4) + U(4));
      T(2) = fa * U(2) + fb * (U(3) + U(1)) + fc * (U(4) + U(2)) + fd * (U(5) + U(3));
      T(3) = fa * U(3) + fb * (U(4) + U(2)) + fc * (U(5) + U(1)) + fd * (U(6) + U(2));
    } else {
      T(1) = 0.0;
      T(2) = fa * U(2) + fb * (U(3) + U(1)) + fc * (U(4) - U(2)) + fd * (U(5) - U(3));
      T(3) = fa * U(3) + fb * (U(4) + U(2)) + fc * (U(5) + U(1)) + fd * (U(6) - U(2));
    }
  } else {
    T(1) = U(1);
    T(2) = a.fia2 * U(1) + a.fib2 * U(2) + a.fic2 * U(3) + a.fid2 * U(4);
    T(3) = a.fia3 * U(1) + a.fib3 * U(2) + a.fic3 * U(3) + a.fid3 * U(4) + a.fie3 * U(5) + a.fif3 * U(6);
  }
  for (int i = 4; i <= nx - 3; ++i)
    T(i) = fa * U(i) + fb * (U(i + 1) + U(i - 1)) + fc * (U(i + 2) + U(i - 2)) + fd * (U(i + 3) + U(i - 3));
  if (cn == 1) {
    if (npaire == 1) {
      T(nx) = fa * U(nx) + fb * (U(nx - 1) + U(nx - 1)) + fc * (U(nx - 2) + U(nx - 2)) + fd * (U(nx - 3) + U(nx - 3));
      T(nx - 1) = fa * U(nx - 1) + fb * (U(nx) + U(nx - 2)) + fc * (U(nx - 1) + U(nx - 3)) + fd * (U(nx - 2) + U(nx - 4));
      T(nx - 2) = fa * U(nx - 2) + fb * (U(nx - 1) + U(nx - 3)) + fc * (U(nx) + U(nx - 4)) + fd * (U(nx - 1) + U(nx - 5));
    } else {
      T(nx) = 0.0;
      T(nx - 1) = fa * U(nx - 1) + fb * (U(nx) + U(nx - 2)) + fc * (-U(nx - 1) + U(nx - 3)) + fd * (-U(nx - 2) + U(nx - 4));
      T(nx - 2) = fa * U(nx - 2) + fb * (U(nx - 1) + U(nx - 3)) + fc * (U(nx) + U(nx - 4)) + fd * (-U(nx - 1) + U(nx - 5));
    }
  } else {
    T(nx) = U(nx);
    T(nx - 1) = a.fiam * U(nx) + a.fibm * U(nx - 1) + a.ficm * U(nx - 2) + a.fidm * U(nx - 3);
    T(nx - 2) = a.fiap * U(nx) + a.fibp * U(nx - 1) + a.ficp * U(nx - 2) + a.fidp * U(nx - 3) + a.fiep * U(nx - 4) +
                a.fifp * U(nx - 5);
  }
}

// Staggered velocity->pressure derivative: src/derive.f90:3796-3907 (derxvp).
void dvp_line(const Axis& a, int npaire, const double* u, double* t) {
  const int nx = a.n, nxm = a.nm;
  const double ac = a.aci6, bc = a.bci6;
  auto wrap = [nx](int i) { return ((i - 1) % nx + nx) % nx + 1; };
  if (a.periodic) {
    for (int i = 1; i <= nx; ++i) T(i) = ac * (U(wrap(i + 1)) - U(i)) + bc * (U(wrap(i + 2)) - U(wrap(i - 1)));
    return;
  }
  if (npaire == 1) {
    T(1) = ac * (U(2) - U(1)) + bc * (U(3) - U(2));
    T(2) = ac * (U(3) - U(2)) + bc * (U(4) - U(1));
    for (int i = 3; i <= nxm - 2; ++i) T(i) = ac * (U(i + 1) - U(i)) + bc * (U(i + 2) - U(i - 1));
    T(nxm - 1) = ac * (U(nxm) - U(nxm - 1)) + bc * (U(nx) - U(nxm - 2));
    T(nxm) = ac * (U(nx) - U(nxm)) + bc * (U(nxm) - U(nxm - 1));
  } else {
    T(1) = ac * (U(2) - U(1)) + bc * (U(3) - 2.0 * U(1) + U(2));
    T(2) = ac * (U(3) - U(2)) + bc * (U(4) - U(1));
    for (int i = 3; i <= nxm - 2; ++i) T(i) = ac * (U(i + 1) - U(i)) + bc * (U(i + 2) - U(i - 1));
    T(nxm - 1) = ac * (U(nxm) - U(nxm - 1)) + bc * (U(nx) - U(nxm - 2));
    T(nxm) = ac * (U(nx) - U(nxm)) + bc * (2.0 * U(nx) - U(nxm) - U(nxm - 1));
  }
}

// Staggered velocity->pressure interpolation: src/derive.f90:3911-4037 (interxvp).
// The non-periodic branch exists only for npaire=1 in the reference.
void ivp_line(const Axis& a, int npaire, const double* u, double* t) {
  const int nx = a.n, nxm = a.nm;
  const double ai = a.aici6, bi = a.bici6, ci = a.cicoef6, di = a.dici6;
  auto wrap = [nx](int i) { return ((i - 1) % nx + nx) % nx + 1; };
  if (a.periodic) {
    for (int i = 1; i <= nx; ++i)
      T(i) = ai * (U(wrap(i + 1)) + U(i)) + bi * (U(wrap(i + 2)) + U(wrap(i - 1))) +
             ci * (U(wrap(i + 3)) + U(wrap(i - 2))) + di * (U(wrap(i + 4)) + U(wrap(i - 3)));
    return;
  }
  (void)npaire;
  T(1) = ai * (U(2) + U(1)) + bi * (U(3) + U(2)) + ci * (U(4) + U(3)) + di * (U(5) + U(4));
  T(2) = ai * (U(3) + U(2)) + bi * (U(4) + U(1)) + ci * (U(5) + U(2)) + di * (U(6) + U(3));
  T(3) = ai * (U(4) + U(3)) + bi * (U(5) + U(2)) + ci * (U(6) + U(1)) + di * (U(7) + U(2));
  for (int i = 4; i <= nxm - 3; ++i)
    T(i) = ai * (U(i + 1) + U(i)) + bi * (U(i + 2) + U(i - 1)) + ci * (U(i + 3) + U(i - 2)) + di * (U(i + 4) + U(i - 3));
  T(nxm - 2) = ai * (U(nxm - 1) + U(nxm - 2)) + bi * (U(nxm) + U(nxm - 3)) + ci * (U(nx) + U(nxm - 4)) +
               di * (U(nxm) + U(nxm - 5));
  T(nxm - 1) = ai * (U(nxm) + U(nxm - 1)) + bi * (U(nx) + U(nxm - 2)) + ci * (U(nxm) + U(nxm - 3)) +
               di * (U(nxm - 1) + U(nxm - 4));
  T(nxm) = ai * (U(nx) + U(nxm)) + bi * (U(nxm) + U(nxm - 1)) + ci * (U(nxm - 1) + U(nxm - 2)) +
           di * (U(nxm - 2) + U(nxm - 3));
}

// Staggered pressure->velocity derivative: src/derive.f90:4041-4122 (derxpv).
// Here u has nm points and t has n points.
void dpv_line(const Axis& a, int npaire, const double* u, double* t) {
  const int nx = a.n;
  const double ac = a.aci6, bc = a.bci6;
  auto wrap = [nx](int i) { return ((i - 1) % nx + nx) % nx + 1; };
  if (a.periodic) {
    for (int i = 1; i <= nx; ++i) T(i) = ac * (U(i) - U(wrap(i - 1))) + bc * (U(wrap(i + 1)) - U(wrap(i - 2)));
    return;
  }
  (void)npaire;
  T(1) = 0.0;
  T(2) = ac * (U(2) - U(1)) + bc * (U(3) - U(1));
  for (int i = 3; i <= nx - 2; ++i) T(i) = ac * (U(i) - U(i - 1)) + bc * (U(i + 1) - U(i - 2));
  T(nx - 1) = ac * (U(nx - 1) - U(nx - 2)) + bc * (U(nx - 1) - U(nx - 3));
  T(nx) = 0.0;
}

// Staggered pressure->velocity interpolation: src/derive.f90:4126-4261 (interxpv).
void ipv_line(const Axis& a, int npaire, const double* u, double* t) {
  const int nx = a.n;
  const double ai = a.aici6, bi = a.bici6, ci = a.cicoef6, di = a.dici6;
  auto wrap = [nx](int i) { return ((i - 1) % nx + nx) % nx + 1; };
  if (a.periodic) {
    for (int i = 1; i <= nx; ++i)
      T(i) = ai * (U(i) + U(wrap(i - 1))) + bi * (U(wrap(i + 1)) + U(wrap(i - 2))) +
             ci * (U(wrap(i + 2)) + U(wrap(i - 3))) + di * (U(wrap(i + 3)) + U(wrap(i - 4)));
    return;
  }
  (void)npaire;
  T(1) = ai * (U(1) + U(1)) + bi * (U(2) + U(2)) + ci * (U(3) + U(3)) + di * (U(4) + U(4));
  T(2) = ai * (U(2) + U(1)) + bi * (U(3) + U(1)) + ci * (U(4) + U(2)) + di * (U(5) + U(3));
  T(3) = ai * (U(3) + U(2)) + bi * (U(4) + U(1)) + ci * (U(5) + U(1)) + di * (U(6) + U(2));
  T(4) = ai * (U(4) + U(3)) + bi * (U(5) + U(2)) + ci * (U(6) + U(1)) + di * (U(7) + U(1));
  for (int i = 5; i <= nx - 4; ++i)
    T(i) = ai * (U(i) + U(i - 1)) + bi * (U(i + 1) + U(i - 2)) + ci * (U(i + 2) + U(i - 3)) + di * (U(i + 3) + U(i - 4));
  T(nx - 3) = ai * (U(nx - 3) + U(nx - 4)) + bi * (U(nx - 2) + U(nx - 5)) + ci * (U(nx - 1) + U(nx - 6)) +
              di * (U(nx - 1) + U(nx - 7));
  T(nx - 2) = ai * (U(nx - 2) + U(nx - 3)) + bi * (U(nx - 1) + U(nx - 4)) + ci * (U(nx - 1) + U(nx - 5)) +
              di * (U(nx - 2) + U(nx - 6));
  T(nx - 1) = ai * (U(nx - 1) + U(nx - 2)) + bi * (U(nx - 1) + U(nx - 3)) + ci * (U(nx - 2) + U(nx - 4)) +
              di * (U(nx - 3) + U(nx - 5));
  T(nx) = ai * (U(nx - 1) + U(nx - 1)) + bi * (U(nx - 2) + U(nx - 2)) + ci * (U(nx - 3) + U(nx - 3)) +
          di * (U(nx - 4) + U(nx - 4));
}

#undef U
#undef T
#undef R

// Sizes and solve factors of one operator on one axis, chosen the way the
// reference's callers choose them (npaire=1 takes the "p" coefficient set).
struct OpPlan {
  int nin, nout;
  const vec *f, *s, *w;
  bool sm;         // periodic Sherman-Morrison correction
  double alpha;    // SM alpha
};

OpPlan plan_op(const Axis& a, int op, int npaire) {
  OpPlan p{};
  p.sm = a.periodic;
  switch (op) {
    case OP_DER1:
      p.nin = p.nout = a.n; p.alpha = a.alfai;
      if (npaire == 1) { p.f = &a.ffp; p.s = &a.fsp; p.w = &a.fwp; } else { p.f = &a.ff; p.s = &a.fs; p.w = &a.fw; }
      break;
    case OP_DER2:
      p.nin = p.nout = a.n; p.alpha = a.alsai;
      if (npaire == 1) { p.f = &a.sfp; p.s = &a.ssp; p.w = &a.swp; } else { p.f = &a.sf; p.s = &a.ss; p.w = &a.sw; }
      break;
    case OP_FIL:
      p.nin = p.nout = a.n; p.alpha = a.fiali;
      if (npaire == 1) { p.f = &a.fiffp; p.s = &a.fifsp; p.w = &a.fifwp; } else { p.f = &a.fiff; p.s = &a.fifs; p.w = &a.fifw; }
      break;
    case OP_DVP:  // derxvp is called with (cfx6,csx6,cwx6) by divergence (src/navier.f90:297)
      p.nin = a.n; p.nout = a.nm; p.alpha = a.alcai6;
      if (npaire == 1) { p.f = &a.cfp6; p.s = &a.csp6; p.w = &a.cwp6; } else { p.f = &a.cf6; p.s = &a.cs6; p.w = &a.cw6; }
      break;
    case OP_IVP:  // interxvp is called with the p set (src/navier.f90:312-313)
      p.nin = a.n; p.nout = a.nm; p.alpha = a.ailcai6;
      if (npaire == 1) { p.f = &a.cifp6; p.s = &a.cisp6; p.w = &a.ciwp6; } else { p.f = &a.cif6; p.s = &a.cis6; p.w = &a.ciw6; }
      break;
    case OP_DPV:  // derxpv(cfip6,csip6,cwip6,cfx6,csx6,cwx6): periodic branch uses the second set
      p.nin = a.nm; p.nout = a.n; p.alpha = a.alcai6;
      if (a.periodic) { p.f = &a.cf6; p.s = &a.cs6; p.w = &a.cw6; }
      else if (npaire == 1) { p.f = &a.cfip6; p.s = &a.csip6; p.w = &a.cwip6; }
      else { p.f = &a.cfi6; p.s = &a.csi6; p.w = &a.cwi6; }
      break;
    case OP_IPV:
      p.nin = a.nm; p.nout = a.n; p.alpha = a.ailcai6;
      if (a.periodic) { p.f = &a.cif6; p.s = &a.cis6; p.w = &a.ciw6; }
      else if (npaire == 1) { p.f = &a.cifip6; p.s = &a.cisip6; p.w = &a.ciwip6; }
      else { p.f = &a.cifi6; p.s = &a.cisi6; p.w = &a.ciwi6; }
      break;
  }
  return p;
}

void apply_line(const Axis& a, int op, int npaire, const OpPlan& p, const double* u, double* t) {
  switch (op) {
    case OP_DER1: der1_line(a, npaire, u, t); break;
    case OP_DER2: der2_line(a, npaire, u, t); break;
    case OP_FIL: fil_line(a, npaire, u, t); break;
    case OP_DVP: dvp_line(a, npaire, u, t); break;
    case OP_IVP: ivp_line(a, npaire, u, t); break;
    case OP_DPV: dpv_line(a, npaire, u, t); break;
    case OP_IPV: ipv_line(a, npaire, u, t); break;
  }
  thomas(t, p.nout, *p.f, *p.s, *p.w);
  if (p.sm) sherman_morrison(t, p.nout, p.alpha, *p.f, *p.s, *p.w);
}

// ---------------------------------------------------------------------------
// FFT (test oracle only): iterative radix-2 for powers of two, direct DFT
// otherwise.  Forward uses exp(-i), the inverse exp(+i), both unnormalised.
// ---------------------------------------------------------------------------
void fft1d(cplx* x, int n, int sign, std::vector<cplx>& work) {
  if (n <= 1) return;
  if ((n & (n - 1)) == 0) {
    for (int i = 1, j = 0; i < n; ++i) {
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(x[i], x[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
      for (int i = 0; i < n; i += len) {
        for (int k = 0; k < len / 2; ++k) {
          const double ang = sign * TWOPI * k / len;
          const cplx w(std::cos(ang), std::sin(ang));
          const cplx a = x[i + k], b = x[i + k + len / 2] * w;
          x[i + k] = a + b;
          x[i + k + len / 2] = a - b;
        }
      }
    }
    return;
  }
  work.assign(n, cplx(0, 0));
  for (int k = 0; k < n; ++k) {
    cplx acc(0, 0);
    for (int m = 0; m < n; ++m) {
      const double ang = sign * TWOPI * (double)((long long)k * m % n) / n;
      acc += x[m] * cplx(std::cos(ang), std::sin(ang));
    }
    work[k] = acc;
  }
  for (int k = 0; k < n; ++k) x[k] = work[k];
}

}  // namespace

// ---------------------------------------------------------------------------
// Oracle context: grid, options and per-axis coefficients.
// ---------------------------------------------------------------------------
struct OxCtx {
  int nx, ny, nz;
  double xlx, yly, zlz;
  Opts opts;
  Axis ax[3];
  // mesh stretching in y (src/stretching.f90:92-270); istret=0 leaves these empty
  int istret = 0;
  double beta = 0, alpha = 0;
  vec yp, ypi, ppy, pp2y, pp4y, ppyi, pp2yi, pp4yi;
  // poisson_000 tables
  vec kx2, ky2, kz2, tx, ty, tz;  // per-axis modified wavenumber^2 and interpolation transfer
  vec sax, sbx, say, sby, saz, sbz;
  // poisson_010 tables (x, z periodic; y non-periodic on nym points)
  vec yky10, yk210, eys10, trx10, try10, trz10;
  // explicit LES (src/les_models.f90): jles 0 none, 1 Smagorinsky, 3 dynamic
  int jles = 0;
  double smagcst = 0.14, maxdsmagcst = 0.3;
  vec del;      // filter width per y row (init_explicit_les)
  Axis axf[3];  // the axes with filter coefficients of alpha = 0 (dynsmag's filter(zero))
};

namespace {

void setup_axis(Axis& a, int n, double len, int ncl1, int ncln, const Opts& o) {
  a.n = n; a.ncl1 = ncl1; a.ncln = ncln;
  a.periodic = (ncl1 == 0 && ncln == 0);
  a.nm = a.periodic ? n : n - 1;
  a.len = len;
  a.d = len / (double)a.nm;  // src/parameters.f90:296-298
  a.d2 = a.d * a.d;
  first_derivative(a, o);
  second_derivative(a, o);
  interpolation(a, o);
  filter_coefficients(a, o.filter_alpha);
}

// Interpolation transfer function at rl = (mode wavenumber) * d, as the
// kxyz assembly of waves writes it (src/poisson.f90:1740-1760).
double transfer(const Axis& a, double rl) {
  const double tt = 2.0 * (a.bici6 * std::cos(rl * 1.5) + a.cicoef6 * std::cos(rl * 2.5) + a.dici6 * std::cos(rl * 3.5));
  const double tt1 = 2.0 * a.aici6 * std::cos(rl * 0.5);
  const double t1 = 1.0 + 2.0 * a.ailcai6 * std::cos(rl);
  return (tt1 + tt) / t1;
}

// Free-slip at both ends (ncl = 1 / 1).
bool slip_axis(const Axis& a) { return a.ncl1 == 1 && a.ncln == 1; }

// Modified wavenumbers of the staggered scheme and the interpolation transfer
// functions: src/poisson.f90:1530-1810 (waves, periodic branches) and the
// kxyz assembly at src/poisson.f90:1688-1724.
void waves_axis(const Axis& a, vec& k2, vec& tr) {
  const int n = a.n;
  k2.assign(n, 0.0);
  tr.assign(n, 0.0);
  vec es(n, 0.0);
  for (int i = 1; i <= n / 2 + 1; ++i) {
    const double w = TWOPI * (i - 1) / n;
    double wp = a.aci6 * 2.0 * a.d * std::sin(w * 0.5) + a.bci6 * 2.0 * a.d * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * a.alcai6 * std::cos(w));
    const double kk = n * wp / a.len;
    k2[i - 1] = kk * kk;
    es[i - 1] = n * w / a.len;
  }
  for (int i = n / 2 + 2; i <= n; ++i) {
    k2[i - 1] = k2[n - i + 1];
    es[i - 1] = es[n - i + 1];
  }
  for (int i = 0; i < n; ++i) {
    const double rl = es[i] * a.d;
    const double tt = 2.0 * (a.bici6 * std::cos(rl * 1.5) + a.cicoef6 * std::cos(rl * 2.5) + a.dici6 * std::cos(rl * 3.5));
    const double tt1 = 2.0 * a.aici6 * std::cos(rl * 0.5);
    const double t1 = 1.0 + 2.0 * a.ailcai6 * std::cos(rl);
    tr[i] = (tt1 + tt) / t1;
  }
}

// abxyz periodic branch: src/poisson.f90:1469-1526.
void abxyz_axis(int n, vec& sa, vec& sb) {
  sa.assign(n, 0.0);
  sb.assign(n, 0.0);
  for (int i = 1; i <= n; ++i) {
    sa[i - 1] = std::sin((double)(i - 1) * PI / (double)n);
    sb[i - 1] = std::cos((double)(i - 1) * PI / (double)n);
  }
}

inline size_t idx3(int i, int j, int k, int nx, int ny) { return (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k); }

// Mesh stretching in y: src/stretching.f90:92-270 (stretching_full) and the
// uniform-mesh defaults of src/variables.f90:1294-1305 (ppy = 1, 2 at
// non-periodic ends).  Fills yp, ypi, ppy, pp2y, pp4y, ppyi, pp2yi, pp4yi and
// the mapping constant alpha.
void stretching_setup(OxCtx& c) {
  const int ny = c.ny;
  const Axis& a = c.ax[1];
  c.yp.assign(ny, 0.0); c.ypi.assign(ny, 0.0);
  c.ppy.assign(ny, 1.0); c.pp2y.assign(ny, 0.0); c.pp4y.assign(ny, 0.0);
  c.ppyi.assign(ny, 1.0); c.pp2yi.assign(ny, 0.0); c.pp4yi.assign(ny, 0.0);
  if (c.istret == 0) {
    for (int j = 0; j < ny; ++j) {
      c.yp[j] = (double)j * a.d;
      c.ypi[j] = ((double)(j + 1) - 0.5) * a.d;
    }
    if (a.ncl1 == 1 || a.ncl1 == 2) c.ppy[0] = 2.0;
    if (a.ncln == 1 || a.ncln == 2) c.ppy[ny - 1] = 2.0;
    return;
  }
  const int istret = c.istret;
  const double beta = c.beta, yly = c.yly;
  const int nym = a.periodic ? ny : ny - 1;
  vec yeta(ny, 0.0), yetai(ny, 0.0);
  const double yinf = -yly / 2.0;
  double den = 2.0 * beta * yinf;
  double xnum = -yinf - std::sqrt(PI * PI * beta * beta + yinf * yinf);
  const double alpha = std::fabs(xnum / den);
  c.alpha = alpha;
  auto mapped = [&](double ye) {
    const double den1 = std::sqrt(alpha * beta + 1.0);
    const double xn = den1 / std::sqrt(alpha / PI) / std::sqrt(beta) / std::sqrt(PI);
    const double dn = 2.0 * std::sqrt(alpha / PI) * std::sqrt(beta) * PI * std::sqrt(PI);
    const double den3 = ((std::sin(PI * ye)) * (std::sin(PI * ye)) / beta / PI) + alpha / PI;
    const double den4 = 2.0 * alpha * beta - std::cos(2.0 * PI * ye) + 1.0;
    const double xnum1 = (std::atan(xn * std::tan(PI * ye))) * den4 / den1 / den3 / dn;
    const double cst = std::sqrt(beta) * PI / (2.0 * std::sqrt(alpha) * std::sqrt(alpha * beta + 1.0));
    double y = 0.0;
    if (istret == 1) {
      if (ye < 0.5) y = xnum1 - cst - yinf;
      if (ye == 0.5) y = 0.0 - yinf;
      if (ye > 0.5) y = xnum1 + cst - yinf;
    } else if (istret == 2) {
      if (ye < 0.5) y = xnum1 - cst + yly;
      if (ye == 0.5) y = 0.0 + yly;
      if (ye > 0.5) y = xnum1 + cst + yly;
    } else {
      if (ye < 0.5) y = (xnum1 - cst + yly) * 2.0;
      if (ye == 0.5) y = (0.0 + yly) * 2.0;
      if (ye > 0.5) y = (xnum1 + cst + yly) * 2.0;
    }
    return y;
  };
  if (alpha != 0.0) {
    c.yp[0] = 0.0;
    yeta[0] = (istret == 1) ? 0.0 : -0.5;
    for (int j = 2; j <= ny; ++j) {
      if (istret == 1) yeta[j - 1] = (double)(j - 1) * (1.0 / (double)nym);
      if (istret == 2) yeta[j - 1] = (double)(j - 1) * (1.0 / (double)nym) - 0.5;
      if (istret == 3) yeta[j - 1] = (double)(j - 1) * (0.5 / (double)nym) - 0.5;
      c.yp[j - 1] = mapped(yeta[j - 1]);
    }
    for (int j = 1; j <= ny; ++j) {
      if (istret == 1) yetai[j - 1] = ((double)j - 0.5) * (1.0 / (double)nym);
      if (istret == 2) yetai[j - 1] = ((double)j - 0.5) * (1.0 / (double)nym) - 0.5;
      if (istret == 3) yetai[j - 1] = ((double)j - 0.5) * (0.5 / (double)nym) - 0.5;
      c.ypi[j - 1] = mapped(yetai[j - 1]);
    }
  } else {
    c.yp[0] = -1.e10;
    for (int j = 2; j <= ny; ++j) {
      yeta[j - 1] = (double)(j - 1) * (1.0 / (double)ny);
      c.yp[j - 1] = -beta * std::cos(PI * yeta[j - 1]) / std::sin(yeta[j - 1] * PI);
    }
    c.ypi[0] = -1.e10;
    for (int j = 2; j <= ny; ++j) {
      yetai[j - 1] = (double)(j - 1) * (1.0 / (double)ny);
      c.ypi[j - 1] = -beta * std::cos(PI * yetai[j - 1]) / std::sin(yetai[j - 1] * PI);
    }
  }
  const double q = (istret == 3) ? 2.0 : 1.0;
  for (int j = 0; j < ny; ++j) {
    c.ppy[j] = yly * (alpha / PI + (1.0 / PI / beta) * std::sin(PI * yeta[j]) * std::sin(PI * yeta[j]));
    c.pp2y[j] = c.ppy[j] * c.ppy[j];
    c.pp4y[j] = (-2.0 / beta * std::cos(PI * yeta[j]) * std::sin(PI * yeta[j]));
    if (istret == 3) c.pp4y[j] = c.pp4y[j] / q;
    c.ppyi[j] = yly * (alpha / PI + (1.0 / PI / beta) * std::sin(PI * yetai[j]) * std::sin(PI * yetai[j]));
    c.pp2yi[j] = c.ppyi[j] * c.ppyi[j];
    c.pp4yi[j] = (-2.0 / beta * std::cos(PI * yetai[j]) * std::sin(PI * yetai[j]));
    if (istret == 3) c.pp4yi[j] = c.pp4yi[j] / q;
  }
}

// Wavenumbers of a non-periodic y axis for poisson_010: src/poisson.f90:1603-1619
// (waves, bcy = 1) and the transfer function of src/poisson.f90:1663-1676.
// yky, yk2, eys have ny (velocity-mesh) entries; the transfer has nym.
void waves_y010(const OxCtx& c, vec& yky, vec& yk2, vec& eys, vec& tr) {
  const Axis& a = c.ax[1];
  const int ny = a.n, nym = a.nm;
  yky.assign(ny, 0.0); yk2.assign(ny, 0.0); eys.assign(ny, 0.0); tr.assign(nym, 0.0);
  for (int j = 1; j <= ny; ++j) {
    const double w = TWOPI * 0.5 * (double)(j - 1) / (double)nym;
    double wp = a.aci6 * 2.0 * a.d * std::sin(w * 0.5) + (a.bci6 * 2.0 * a.d) * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * a.alcai6 * std::cos(w));
    yky[j - 1] = (c.istret == 0) ? (double)nym * wp / c.yly : (double)nym * wp;
    eys[j - 1] = (double)nym * w / c.yly;
    const double t = (double)nym * wp / c.yly;
    yk2[j - 1] = t * t;
  }
  yky[0] = 0.0; eys[0] = 0.0; yk2[0] = 0.0;
  for (int j = 0; j < nym; ++j) {
    const double rl = eys[j] * a.d;
    const double tt = 2.0 * (a.bici6 * std::cos(rl * 1.5) + a.cicoef6 * std::cos(rl * 2.5) + a.dici6 * std::cos(rl * 3.5));
    const double tt1 = 2.0 * a.aici6 * std::cos(rl * 0.5);
    const double t1 = 1.0 + 2.0 * a.ailcai6 * std::cos(rl);
    tr[j] = (tt1 + tt) / t1;
  }
}

// abxyz, non-periodic branch: src/poisson.f90:1489-1496.
void abxyz_half(int n, vec& sa, vec& sb) {
  sa.assign(n, 0.0);
  sb.assign(n, 0.0);
  for (int i = 1; i <= n; ++i) {
    sa[i - 1] = std::sin((double)(i - 1) * PI * 0.5 / (double)n);
    sb[i - 1] = std::cos((double)(i - 1) * PI * 0.5 / (double)n);
  }
}

// Apply operator `op` along `axis` to the 3-D field u (dims nin along the axis),
// writing t (dims nout along the axis).  dims[] are the input dims.
void apply3d(const OxCtx& c, int axis, int op, int npaire, const double* u, double* t, const int dims[3],
             const double* pp, const Axis* override_axis = nullptr) {
  const Axis& a = override_axis ? *override_axis : c.ax[axis];
  const OpPlan p = plan_op(a, op, npaire);
  int din[3] = {dims[0], dims[1], dims[2]};
  int dout[3] = {dims[0], dims[1], dims[2]};
  dout[axis] = p.nout;
  const int o1 = (axis == 0) ? 1 : 0, o2 = (axis == 2) ? 1 : 2;
  const int n1 = din[o1], n2 = din[o2];
#pragma omp parallel
  {
    vec lu(p.nin), lt(p.nout);
#pragma omp for collapse(2) schedule(static)
    for (int b = 0; b < n2; ++b)
      for (int aa = 0; aa < n1; ++aa) {
        int ii[3];
        ii[o1] = aa; ii[o2] = b;
        for (int m = 0; m < p.nin; ++m) {
          ii[axis] = m;
          lu[m] = u[idx3(ii[0], ii[1], ii[2], din[0], din[1])];
        }
        apply_line(a, op, npaire, p, lu.data(), lt.data());
        for (int m = 0; m < p.nout; ++m) {
          ii[axis] = m;
          double v = lt[m];
          if (pp) v = v * pp[m];
          t[idx3(ii[0], ii[1], ii[2], dout[0], dout[1])] = v;
        }
      }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Periodic Poisson solve: src/poisson.f90:298-410 (poisson_000).
// The forward transform follows 2DECOMP's PHYSICAL_IN_Z convention: r2c along
// z (nz/2+1 modes), then complex transforms along y and x; spectral array
// (nx, ny, nz/2+1).
// ---------------------------------------------------------------------------
static void poisson_000(const OxCtx& c, double* rhs) {
  const int nx = c.nx, ny = c.ny, nz = c.nz, nz2 = nz / 2 + 1;
  std::vector<cplx> cw((size_t)nx * ny * nz2);
  auto CW = [&](int i, int j, int k) -> cplx& { return cw[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)]; };
#pragma omp parallel
  {
    std::vector<cplx> line, work;
#pragma omp for collapse(2)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        line.assign(nz, cplx(0, 0));
        for (int k = 0; k < nz; ++k) line[k] = cplx(rhs[idx3(i, j, k, nx, ny)], 0.0);
        fft1d(line.data(), nz, -1, work);
        for (int k = 0; k < nz2; ++k) CW(i, j, k) = line[k];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int i = 0; i < nx; ++i) {
        line.resize(ny);
        for (int j = 0; j < ny; ++j) line[j] = CW(i, j, k);
        fft1d(line.data(), ny, -1, work);
        for (int j = 0; j < ny; ++j) CW(i, j, k) = line[j];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int j = 0; j < ny; ++j) {
        line.resize(nx);
        for (int i = 0; i < nx; ++i) line[i] = CW(i, j, k);
        fft1d(line.data(), nx, -1, work);
        for (int i = 0; i < nx; ++i) CW(i, j, k) = line[i];
      }
  }
  const double eps = 1.0e-16;
#pragma omp parallel for collapse(2)
  for (int k = 0; k < nz2; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        cplx v = CW(i, j, k);
        double re = v.real() / (double)nx / (double)ny / (double)nz;
        double im = v.imag() / (double)nx / (double)ny / (double)nz;
        double t1, t2;
        // forward shifts (z, y, x)
        t1 = re; t2 = im;
        re = t1 * c.sbz[k] + t2 * c.saz[k]; im = t2 * c.sbz[k] - t1 * c.saz[k];
        t1 = re; t2 = im;
        re = t1 * c.sby[j] + t2 * c.say[j]; im = t2 * c.sby[j] - t1 * c.say[j];
        if (j + 1 > ny / 2 + 1) { re = -re; im = -im; }
        t1 = re; t2 = im;
        re = t1 * c.sbx[i] + t2 * c.sax[i]; im = t2 * c.sbx[i] - t1 * c.sax[i];
        if (i + 1 > nx / 2 + 1) { re = -re; im = -im; }
        // kxyz = xk2*(ty*tz)^2 + yk2*(tx*tz)^2 + zk2*(tx*ty)^2 (both parts equal)
        const double pyz = c.ty[j] * c.tz[k], pxz = c.tx[i] * c.tz[k], pxy = c.tx[i] * c.ty[j];
        const double kk = c.kx2[i] * (pyz * pyz) + c.ky2[j] * (pxz * pxz) + c.kz2[k] * (pxy * pxy);
        if ((kk < eps) || (kk < eps)) {
          re = 0.0; im = 0.0;
        } else {
          re = re / (-kk); im = im / (-kk);
        }
        // backward shifts
        t1 = re; t2 = im;
        re = t1 * c.sbz[k] - t2 * c.saz[k]; im = -t2 * c.sbz[k] - t1 * c.saz[k];
        t1 = re; t2 = im;
        re = t1 * c.sby[j] + t2 * c.say[j]; im = t2 * c.sby[j] - t1 * c.say[j];
        if (j + 1 > ny / 2 + 1) { re = -re; im = -im; }
        t1 = re; t2 = im;
        re = t1 * c.sbx[i] + t2 * c.sax[i]; im = -t2 * c.sbx[i] + t1 * c.sax[i];
        if (i + 1 > nx / 2 + 1) { re = -re; im = -im; }
        CW(i, j, k) = cplx(re, im);
      }
#pragma omp parallel
  {
    std::vector<cplx> line, work;
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int j = 0; j < ny; ++j) {
        line.resize(nx);
        for (int i = 0; i < nx; ++i) line[i] = CW(i, j, k);
        fft1d(line.data(), nx, +1, work);
        for (int i = 0; i < nx; ++i) CW(i, j, k) = line[i];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int i = 0; i < nx; ++i) {
        line.resize(ny);
        for (int j = 0; j < ny; ++j) line[j] = CW(i, j, k);
        fft1d(line.data(), ny, +1, work);
        for (int j = 0; j < ny; ++j) CW(i, j, k) = line[j];
      }
#pragma omp for collapse(2)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        // c2r along z: Hermitian extension of the half spectrum, real part taken.
        line.assign(nz, cplx(0, 0));
        for (int k = 0; k < nz2; ++k) line[k] = CW(i, j, k);
        for (int k = nz2; k < nz; ++k) line[k] = std::conj(CW(i, j, nz - k));
        line[0] = cplx(line[0].real(), 0.0);
        if (nz % 2 == 0) line[nz / 2] = cplx(line[nz / 2].real(), 0.0);
        fft1d(line.data(), nz, +1, work);
        for (int k = 0; k < nz; ++k) rhs[idx3(i, j, k, nx, ny)] = line[k].real();
      }
  }
}

// ---------------------------------------------------------------------------
// Poisson solve with x and z periodic and y non-periodic (Neumann):
// src/poisson.f90:665-1013 (poisson_010), spectral array (nx, nym, nz/2+1)
// as 2DECOMP's PHYSICAL_IN_Z transform leaves it.
// ---------------------------------------------------------------------------

// Pentadiagonal systems of src/poisson.f90:1814-2113 (matrice_refinement,
// istret = 1 or 2, bcz = 0).  With x and z periodic every coefficient of the
// reference is cx_one_one times a real number, so the real value is kept and
// serves both the real and the imaginary solve.  Layout: d[q][i + nx*(m + nh*k)].
struct Penta {
  int nx = 0, nh = 0, nk = 0;
  vec d[5];
  double& at(int q, int i, int m, int k) { return d[q][(size_t)i + (size_t)nx * ((size_t)m + (size_t)nh * k)]; }
  double at(int q, int i, int m, int k) const { return d[q][(size_t)i + (size_t)nx * ((size_t)m + (size_t)nh * k)]; }
};

void matrice_refinement(const OxCtx& c, Penta& A, Penta& A2) {
  const int nx = c.nx, nym = c.ax[1].nm, nz2 = c.nz / 2 + 1, nh = nym / 2;
  for (Penta* P : {&A, &A2}) {
    P->nx = nx; P->nh = nh; P->nk = nz2;
    for (int q = 0; q < 5; ++q) P->d[q].assign((size_t)nx * nh * nz2, 0.0);
  }
  const double alpha = c.alpha, beta = c.beta;
  const double xa0 = alpha / PI + 0.5 / beta / PI;
  const double xa1 = (c.istret == 1) ? 1.0 / 4.0 / beta / PI : -(1.0 / 4.0 / beta / PI);
  const double xa0_2 = xa0 * xa0, xa1_2 = xa1 * xa1, xa01 = xa0 * xa1, xa0p1_2 = (xa0 + xa1) * (xa0 + xa1);
  const vec &kx2 = c.kx2, &kz2 = c.kz2, &tx = c.trx10, &tz = c.trz10, &ty = c.try10, &yky = c.yky10;
  auto ty2 = [&](int j1) { return ty[j1 - 1] * ty[j1 - 1]; };  // transy_rl2, 1-based
  vec c1(nh + 2), c2(nh + 2);                                   // cw22 / cw2, 1-based
  for (int k = 0; k < nz2; ++k)
    for (int i = 0; i < nx; ++i) {
      const double tx2 = tx[i] * tx[i], tz2 = tz[k] * tz[k];
      for (int j = 1; j <= nh; ++j) {
        c1[j] = tx[i] * (yky[2 * j - 2] * tz[k]);
        c2[j] = tx[i] * (yky[2 * j - 1] * tz[k]);
      }
      auto diag = [&](int jy, double cc, double a2c, double nb) {
        return -(kx2[i] * ty2(jy) * tz2 + kz2[k] * ty2(jy) * tx2 + a2c * (cc * cc) + xa1_2 * cc * nb);
      };
      // main diagonal
      for (int j = 2; j <= nh - 1; ++j) {
        A.at(2, i, j - 1, k) = diag(2 * j - 1, c1[j], xa0_2, c1[j - 1] + c1[j + 1]);
        A2.at(2, i, j - 1, k) = diag(2 * j, c2[j], xa0_2, c2[j - 1] + c2[j + 1]);
      }
      A.at(2, i, 0, k) = diag(1, c1[1], xa0_2, c1[2]);
      A.at(2, i, nh - 1, k) = diag(2 * nh - 1, c1[nh], xa0_2, c1[nh - 1]);
      A2.at(2, i, 0, k) = diag(2, c2[1], xa0_2 - xa1_2, c2[2]);
      A2.at(2, i, nh - 1, k) = diag(2 * nh, c2[nh], xa0p1_2, c2[nh - 1]);
      // super-diagonal +1
      for (int j = 2; j <= nh - 1; ++j) {
        A.at(3, i, j - 1, k) = xa01 * (c1[j + 1] * (c1[j] + c1[j + 1]));
        A2.at(3, i, j - 1, k) = xa01 * (c2[j + 1] * (c2[j] + c2[j + 1]));
      }
      A.at(3, i, 0, k) = 2.0 * xa01 * (c1[1] * c1[2] + c1[2] * c1[2]);
      A2.at(3, i, 0, k) = (xa0 - xa1) * xa1 * (c2[1] * c2[2]) + xa0 * xa1 * (c2[2] * c2[2]);
      A2.at(3, i, nh - 2, k) = xa0 * xa1 * c2[nh - 1] * c2[nh] + (xa0 + xa1) * xa1 * (c2[nh] * c2[nh]);
      A2.at(3, i, nh - 1, k) = 0.0;
      // super-diagonal +2
      for (int j = 1; j <= nh - 2; ++j) {
        A.at(4, i, j - 1, k) = xa1_2 * (-(c1[j + 1] * c1[j + 2]));
        A2.at(4, i, j - 1, k) = xa1_2 * (-(c2[j + 1] * c2[j + 2]));
      }
      A.at(4, i, 0, k) = 2.0 * A.at(4, i, 0, k);
      A.at(4, i, nh - 2, k) = 0.0; A.at(4, i, nh - 1, k) = 0.0;
      A2.at(4, i, nh - 2, k) = 0.0; A2.at(4, i, nh - 1, k) = 0.0;
      // sub-diagonal -1
      for (int j = 2; j <= nh; ++j) {
        A.at(1, i, j - 1, k) = xa01 * (c1[j - 1] * (c1[j] + c1[j - 1]));
        A2.at(1, i, j - 1, k) = xa01 * (c2[j - 1] * (c2[j] + c2[j - 1]));
      }
      A.at(1, i, 0, k) = 0.0; A2.at(1, i, 0, k) = 0.0;
      A2.at(1, i, 1, k) = xa0 * xa1 * (c2[2] * c2[1]) + (xa0 + xa1) * xa1 * (c2[1] * c2[1]);
      A2.at(1, i, nh - 1, k) = (xa0 + xa1) * xa1 * (c2[nh] * c2[nh - 1]) + xa0 * xa1 * (c2[nh - 1] * c2[nh - 1]);
      // sub-diagonal -2
      for (int j = 3; j <= nh; ++j) {
        A.at(0, i, j - 1, k) = xa1_2 * (-(c1[j - 1] * c1[j - 2]));
        A2.at(0, i, j - 1, k) = xa1_2 * (-(c2[j - 1] * c2[j - 2]));
      }
      A.at(0, i, 0, k) = 0.0; A.at(0, i, 1, k) = 0.0;
      A2.at(0, i, 0, k) = 0.0; A2.at(0, i, 1, k) = 0.0;
      // the (kx, kz) = (0, 0) line: pin the first odd mode (no singular matrix)
      if (kx2[i] == 0.0 && kz2[k] == 0.0) {
        A.at(2, i, 0, k) = 1.0; A.at(3, i, 0, k) = 0.0; A.at(4, i, 0, k) = 0.0;
      }
    }
}

// src/tools.f90:1225-1362 (inversion5_v1): banded Gaussian elimination of the
// pentadiagonal systems, real and imaginary parts separately (here with the
// same real matrix).  Loop order and the epsilon guards follow the reference;
// the pivots of the forward sweep are non-zero for these matrices.
void inversion5_v1(const Penta& Ain, std::vector<cplx>& e, int nx, int nk) {
  Penta a = Ain;
  const int nh = a.nh;
  const double eps = 1.0e-16;
  auto E = [&](int i, int m, int k) -> cplx& { return e[(size_t)i + (size_t)nx * ((size_t)m + (size_t)nh * k)]; };
  vec sr((size_t)nx * nk);
  double tmp1 = 0, tmp2 = 0;
  const int ja[2] = {3, 2}, jb[2] = {4, 3};  // 1-based diagonal indices
  for (int m = 1; m <= nh - 2; ++m)
    for (int ii = 1; ii <= 2; ++ii) {
      const int mi = m + ii;
      for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nx; ++j) {
          const double piv = a.at(2, j, m - 1, k);
          if (piv != 0.0) tmp1 = a.at(2 - ii, j, mi - 1, k) / piv;
          if (piv != 0.0) tmp2 = a.at(2 - ii, j, mi - 1, k) / piv;
          sr[(size_t)j + (size_t)nx * k] = tmp1;
          const cplx em = E(j, m - 1, k), emi = E(j, mi - 1, k);
          E(j, mi - 1, k) = cplx(emi.real() - tmp1 * em.real(), emi.imag() - tmp2 * em.imag());
        }
      for (int jc = ja[ii - 1]; jc <= jb[ii - 1]; ++jc)
        for (int k = 0; k < nk; ++k)
          for (int j = 0; j < nx; ++j)
            a.at(jc - 1, j, mi - 1, k) =
                a.at(jc - 1, j, mi - 1, k) - sr[(size_t)j + (size_t)nx * k] * a.at(jc + ii - 1, j, m - 1, k);
    }
  for (int k = 0; k < nk; ++k)
    for (int j = 0; j < nx; ++j) {
      const double p1 = a.at(2, j, nh - 2, k);
      const double s = (std::fabs(p1) > eps) ? a.at(1, j, nh - 1, k) / p1 : 0.0;
      const double b1 = a.at(2, j, nh - 1, k) - s * a.at(3, j, nh - 2, k);
      const cplx en = E(j, nh - 1, k), en1 = E(j, nh - 2, k);
      double t3r = 0, t3i = 0;
      if (std::fabs(b1) > eps) {
        const double t1 = s / b1;
        t3r = en.real() / b1 - t1 * en1.real();
        t3i = en.imag() / b1 - t1 * en1.imag();
      }
      E(j, nh - 1, k) = cplx(t3r, t3i);
      const double r = (std::fabs(p1) > eps) ? 1.0 / p1 : 0.0;
      const double a1 = a.at(3, j, nh - 2, k) * r;
      const cplx enew = E(j, nh - 1, k);
      E(j, nh - 2, k) = cplx(en1.real() * r - a1 * enew.real(), en1.imag() * r - a1 * enew.imag());
    }
  for (int i = nh - 2; i >= 1; --i)
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nx; ++j) {
        const double p = a.at(2, j, i - 1, k);
        const double r = (std::fabs(p) > eps) ? 1.0 / p : 0.0;
        const double a1 = a.at(3, j, i - 1, k) * r;
        const double b1 = a.at(4, j, i - 1, k) * r;
        const cplx e0 = E(j, i - 1, k), e1 = E(j, i, k), e2 = E(j, i + 1, k);
        E(j, i - 1, k) = cplx(e0.real() * r - a1 * e1.real() - b1 * e2.real(),
                              e0.imag() * r - a1 * e1.imag() - b1 * e2.imag());
      }
}

static void poisson_010(const OxCtx& c, double* rhs) {
  const int nx = c.nx, ny = c.ax[1].nm, nz = c.nz, nz2 = nz / 2 + 1, nh = ny / 2;
  const size_t N = (size_t)nx * ny * nz;
  // even/odd reorder in y (src/poisson.f90:688-698)
  {
    vec t(rhs, rhs + N);
    for (int k = 0; k < nz; ++k)
      for (int i = 0; i < nx; ++i) {
        for (int j = 1; j <= ny / 2; ++j) rhs[idx3(i, j - 1, k, nx, ny)] = t[idx3(i, 2 * (j - 1), k, nx, ny)];
        for (int j = ny / 2 + 1; j <= ny; ++j) rhs[idx3(i, j - 1, k, nx, ny)] = t[idx3(i, 2 * ny - 2 * j + 1, k, nx, ny)];
      }
  }
  std::vector<cplx> cw((size_t)nx * ny * nz2);
  auto CW = [&](int i, int j, int k) -> cplx& { return cw[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)]; };
#pragma omp parallel
  {
    std::vector<cplx> line, work;
#pragma omp for collapse(2)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        line.assign(nz, cplx(0, 0));
        for (int k = 0; k < nz; ++k) line[k] = cplx(rhs[idx3(i, j, k, nx, ny)], 0.0);
        fft1d(line.data(), nz, -1, work);
        for (int k = 0; k < nz2; ++k) CW(i, j, k) = line[k];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int i = 0; i < nx; ++i) {
        line.resize(ny);
        for (int j = 0; j < ny; ++j) line[j] = CW(i, j, k);
        fft1d(line.data(), ny, -1, work);
        for (int j = 0; j < ny; ++j) CW(i, j, k) = line[j];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int j = 0; j < ny; ++j) {
        line.resize(nx);
        for (int i = 0; i < nx; ++i) line[i] = CW(i, j, k);
        fft1d(line.data(), nx, -1, work);
        for (int i = 0; i < nx; ++i) CW(i, j, k) = line[i];
      }
  }
  for (auto& v : cw) v = cplx(v.real() / (double)nx / (double)ny / (double)nz, v.imag() / (double)nx / (double)ny / (double)nz);
  // post-processing in z and x
  for (int k = 0; k < nz2; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        cplx& v = CW(i, j, k);
        double t1 = v.real(), t2 = v.imag();
        v = cplx(t1 * c.sbz[k] + t2 * c.saz[k], t2 * c.sbz[k] - t1 * c.saz[k]);
        t1 = v.real(); t2 = v.imag();
        v = cplx(t1 * c.sbx[i] + t2 * c.sax[i], t2 * c.sbx[i] - t1 * c.sax[i]);
        if (i + 1 > nx / 2 + 1) v = -v;
      }
  // post-processing in y (src/poisson.f90:764-785)
  std::vector<cplx> cb(cw.size());
  auto CB = [&](int i, int j, int k) -> cplx& { return cb[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)]; };
  for (int k = 0; k < nz2; ++k)
    for (int i = 0; i < nx; ++i) {
      CB(i, 0, k) = CW(i, 0, k);
      for (int j = 2; j <= ny; ++j) {
        const double t1 = CW(i, j - 1, k).real(), t2 = CW(i, j - 1, k).imag();
        const double t3 = CW(i, ny - j + 1, k).real(), t4 = CW(i, ny - j + 1, k).imag();
        const double by = c.sby[j - 1], ay = c.say[j - 1];
        const double x1 = t1 * by, x2 = t1 * ay, x3 = t2 * by, x4 = t2 * ay;
        const double x5 = t3 * by, x6 = t3 * ay, x7 = t4 * by, x8 = t4 * ay;
        CB(i, j - 1, k) = cplx(0.5 * (x1 + x4 + x5 - x8), 0.5 * (-x2 + x3 + x6 + x7));
      }
    }
  if (c.istret == 0) {
    const double eps = 1.0e-16;
    for (int k = 0; k < nz2; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double pyz = c.try10[j] * c.trz10[k], pxz = c.trx10[i] * c.trz10[k], pxy = c.trx10[i] * c.try10[j];
          const double kk = c.kx2[i] * (pyz * pyz) + c.yk210[j] * (pxz * pxz) + c.kz2[k] * (pxy * pxy);
          cplx& v = CB(i, j, k);
          if (std::fabs(kk) < eps) v = cplx(0.0, 0.0);
          else v = cplx(v.real() / (-kk), v.imag() / (-kk));
        }
  } else {
    Penta A, A2;
    matrice_refinement(c, A, A2);
    std::vector<cplx> odd((size_t)nx * nh * nz2), even(odd.size());
    for (int k = 0; k < nz2; ++k)
      for (int j = 1; j <= nh; ++j)
        for (int i = 0; i < nx; ++i) {
          odd[(size_t)i + (size_t)nx * ((size_t)(j - 1) + (size_t)nh * k)] = CB(i, 2 * j - 2, k);
          even[(size_t)i + (size_t)nx * ((size_t)(j - 1) + (size_t)nh * k)] = CB(i, 2 * j - 1, k);
        }
    inversion5_v1(A, odd, nx, nz2);
    inversion5_v1(A2, even, nx, nz2);
    for (int k = 0; k < nz2; ++k)
      for (int j = 1; j <= nh; ++j)
        for (int i = 0; i < nx; ++i) {
          CB(i, 2 * j - 2, k) = odd[(size_t)i + (size_t)nx * ((size_t)(j - 1) + (size_t)nh * k)];
          CB(i, 2 * j - 1, k) = even[(size_t)i + (size_t)nx * ((size_t)(j - 1) + (size_t)nh * k)];
        }
  }
  for (int j = 0; j < ny; ++j) CB(nx / 2, j, nz / 2) = cplx(0.0, 0.0);
  // backward post-processing in y (src/poisson.f90:907-929)
  for (int k = 0; k < nz2; ++k)
    for (int i = 0; i < nx; ++i) {
      CW(i, 0, k) = CB(i, 0, k);
      for (int j = 2; j <= ny; ++j) {
        const double t1 = CB(i, j - 1, k).real(), t2 = CB(i, j - 1, k).imag();
        const double t3 = CB(i, ny - j + 1, k).real(), t4 = CB(i, ny - j + 1, k).imag();
        const double by = c.sby[j - 1], ay = c.say[j - 1];
        const double x1 = t1 * by, x2 = t1 * ay, x3 = t2 * by, x4 = t2 * ay;
        const double x5 = t3 * by, x6 = t3 * ay, x7 = t4 * by, x8 = t4 * ay;
        CW(i, j - 1, k) = cplx(x1 - x4 + x6 + x7, -(-x2 - x3 + x5 - x8));
      }
    }
  // backward post-processing in x and z
  for (int k = 0; k < nz2; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        cplx& v = CW(i, j, k);
        double t1 = v.real(), t2 = v.imag();
        v = cplx(t1 * c.sbx[i] - t2 * c.sax[i], t2 * c.sbx[i] + t1 * c.sax[i]);
        if (i + 1 > nx / 2 + 1) v = -v;
        t1 = v.real(); t2 = v.imag();
        v = cplx(t1 * c.sbz[k] - t2 * c.saz[k], t2 * c.sbz[k] + t1 * c.saz[k]);
      }
#pragma omp parallel
  {
    std::vector<cplx> line, work;
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int j = 0; j < ny; ++j) {
        line.resize(nx);
        for (int i = 0; i < nx; ++i) line[i] = CW(i, j, k);
        fft1d(line.data(), nx, +1, work);
        for (int i = 0; i < nx; ++i) CW(i, j, k) = line[i];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < nz2; ++k)
      for (int i = 0; i < nx; ++i) {
        line.resize(ny);
        for (int j = 0; j < ny; ++j) line[j] = CW(i, j, k);
        fft1d(line.data(), ny, +1, work);
        for (int j = 0; j < ny; ++j) CW(i, j, k) = line[j];
      }
#pragma omp for collapse(2)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        line.assign(nz, cplx(0, 0));
        for (int k = 0; k < nz2; ++k) line[k] = CW(i, j, k);
        for (int k = nz2; k < nz; ++k) line[k] = std::conj(CW(i, j, nz - k));
        line[0] = cplx(line[0].real(), 0.0);
        if (nz % 2 == 0) line[nz / 2] = cplx(line[nz / 2].real(), 0.0);
        fft1d(line.data(), nz, +1, work);
        for (int k = 0; k < nz; ++k) rhs[idx3(i, j, k, nx, ny)] = line[k].real();
      }
  }
  // inverse reorder (src/poisson.f90:995-1006)
  {
    vec t(rhs, rhs + N);
    for (int k = 0; k < nz; ++k)
      for (int i = 0; i < nx; ++i)
        for (int j = 1; j <= ny / 2; ++j) {
          rhs[idx3(i, 2 * j - 2, k, nx, ny)] = t[idx3(i, j - 1, k, nx, ny)];
          rhs[idx3(i, 2 * j - 1, k, nx, ny)] = t[idx3(i, ny - j, k, nx, ny)];
        }
  }
}

// ---------------------------------------------------------------------------
// Explicit LES: src/les_models.f90
// ---------------------------------------------------------------------------
struct StrainT {
  vec sxx, syy, szz, sxy, sxz, syz, srt;
};

// Strain-rate tensor and srt = S:S of smag (src/les_models.f90:168-270).
static void les_strain(const OxCtx& c, const vec& ux, const vec& uy, const vec& uz, StrainT& S) {
  const size_t N = ux.size();
  const int dims[3] = {c.nx, c.ny, c.nz};
  const double* ppy = (c.istret != 0) ? c.ppy.data() : nullptr;
  vec gxx(N), gyx(N), gzx(N), gxy(N), gyy(N), gzy(N), gxz(N), gyz(N), gzz(N);
  apply3d(c, 0, OP_DER1, 0, ux.data(), gxx.data(), dims, nullptr);
  apply3d(c, 0, OP_DER1, 1, uy.data(), gyx.data(), dims, nullptr);
  apply3d(c, 0, OP_DER1, 1, uz.data(), gzx.data(), dims, nullptr);
  apply3d(c, 1, OP_DER1, 1, ux.data(), gxy.data(), dims, ppy);
  apply3d(c, 1, OP_DER1, 0, uy.data(), gyy.data(), dims, ppy);
  apply3d(c, 1, OP_DER1, 1, uz.data(), gzy.data(), dims, ppy);
  apply3d(c, 2, OP_DER1, 1, ux.data(), gxz.data(), dims, nullptr);
  apply3d(c, 2, OP_DER1, 1, uy.data(), gyz.data(), dims, nullptr);
  apply3d(c, 2, OP_DER1, 0, uz.data(), gzz.data(), dims, nullptr);
  S.sxx = gxx; S.syy = gyy; S.szz = gzz;
  S.sxy.resize(N); S.syz.resize(N); S.sxz.resize(N); S.srt.resize(N);
  for (size_t m = 0; m < N; ++m) {
    S.sxy[m] = 0.5 * (gxy[m] + gyx[m]);
    S.syz[m] = 0.5 * (gyz[m] + gzy[m]);
    S.sxz[m] = 0.5 * (gzx[m] + gxz[m]);
  }
  for (size_t m = 0; m < N; ++m)
    S.srt[m] = S.sxx[m] * S.sxx[m] + S.syy[m] * S.syy[m] + S.szz[m] * S.szz[m] + 2.0 * S.sxy[m] * S.sxy[m] +
               2.0 * S.sxz[m] * S.sxz[m] + 2.0 * S.syz[m] * S.syz[m];
}

inline int jrow(size_t m, int nx, int ny) { return (int)((m / (size_t)nx) % (size_t)ny); }

// smag (src/les_models.f90:168-331), itype != abl: nut = (Cs del)^2 sqrt(2 S:S).
static void les_smag(const OxCtx& c, const StrainT& S, vec& nut) {
  const size_t N = S.srt.size();
  nut.assign(N, 0.0);
  for (size_t m = 0; m < N; ++m) {
    const double length = c.smagcst * c.del[jrow(m, c.nx, c.ny)];
    nut[m] = (length * length) * std::sqrt(2.0 * S.srt[m]);
  }
}

// One filter pass of dynsmag (filx / fily / filz with the alpha = 0 filter).
static void les_fil(const OxCtx& c, int axis, int npaire, const vec& u, vec& t) {
  const int dims[3] = {c.nx, c.ny, c.nz};
  t.resize(u.size());
  apply3d(c, axis, OP_FIL, npaire, u.data(), t.data(), dims, nullptr, &c.axf[axis]);
}
// x, then y, then z filtering with one parity per direction.
static void les_fil3(const OxCtx& c, const vec& u, int px, int py, int pz, vec& out) {
  vec a, b;
  les_fil(c, 0, px, u, a);
  les_fil(c, 1, py, a, b);
  les_fil(c, 2, pz, b, out);
}

// dynsmag (src/les_models.f90:333-903), no IBM.  Returns nut; S receives the
// strain tensor of the unfiltered velocity (used by the SGS divergence).
static void les_dynsmag(const OxCtx& c, const vec& ux, const vec& uy, const vec& uz, vec& nut, StrainT& S) {
  const size_t N = ux.size();
  vec uxx(N), uyy(N), uzz(N), uxy(N), uxz(N), uyz(N);
  for (size_t m = 0; m < N; ++m) {
    uxx[m] = ux[m] * ux[m]; uyy[m] = uy[m] * uy[m]; uzz[m] = uz[m] * uz[m];
    uxy[m] = ux[m] * uy[m]; uxz[m] = ux[m] * uz[m]; uyz[m] = uy[m] * uz[m];
  }
  vec uxf, uyf, uzf, uxxf, uyyf, uzzf, uxyf, uxzf, uyzf;
  les_fil3(c, ux, 0, 1, 1, uxf);
  les_fil3(c, uy, 1, 0, 1, uyf);
  les_fil3(c, uz, 1, 1, 0, uzf);
  les_fil3(c, uxx, 1, 1, 1, uxxf);
  les_fil3(c, uyy, 1, 1, 1, uyyf);
  les_fil3(c, uzz, 1, 1, 1, uzzf);
  les_fil3(c, uxy, 0, 0, 1, uxyf);
  les_fil3(c, uxz, 0, 1, 0, uxzf);
  les_fil3(c, uyz, 1, 0, 0, uyzf);
  vec lxx(N), lyy(N), lzz(N), lxy(N), lxz(N), lyz(N);
  for (size_t m = 0; m < N; ++m) {
    lxx[m] = uxxf[m] - uxf[m] * uxf[m];
    lyy[m] = uyyf[m] - uyf[m] * uyf[m];
    lzz[m] = uzzf[m] - uzf[m] * uzf[m];
    lxy[m] = uxyf[m] - uxf[m] * uyf[m];
    lxz[m] = uxzf[m] - uxf[m] * uzf[m];
    lyz[m] = uyzf[m] - uyf[m] * uzf[m];
  }
  StrainT Sf;
  les_strain(c, uxf, uyf, uzf, Sf);
  les_strain(c, ux, uy, uz, S);
  vec bb[6], aa[6];
  const vec* sf[6] = {&Sf.sxx, &Sf.syy, &Sf.szz, &Sf.sxy, &Sf.sxz, &Sf.syz};
  const vec* su[6] = {&S.sxx, &S.syy, &S.szz, &S.sxy, &S.sxz, &S.syz};
  for (int q = 0; q < 6; ++q) { bb[q].resize(N); aa[q].resize(N); }
  for (size_t m = 0; m < N; ++m) {
    const double mf = std::sqrt(2.0 * (Sf.sxx[m] * Sf.sxx[m] + Sf.syy[m] * Sf.syy[m] + Sf.szz[m] * Sf.szz[m] +
                                       2.0 * Sf.sxy[m] * Sf.sxy[m] + 2.0 * Sf.sxz[m] * Sf.sxz[m] +
                                       2.0 * Sf.syz[m] * Sf.syz[m]));
    const double mu = std::sqrt(2.0 * (S.sxx[m] * S.sxx[m] + S.syy[m] * S.syy[m] + S.szz[m] * S.szz[m] +
                                       2.0 * S.sxy[m] * S.sxy[m] + 2.0 * S.sxz[m] * S.sxz[m] +
                                       2.0 * S.syz[m] * S.syz[m]));
    const double dl = c.del[jrow(m, c.nx, c.ny)];
    for (int q = 0; q < 6; ++q) {
      bb[q][m] = -2.0 * mf * (*sf[q])[m];
      aa[q][m] = -2.0 * mu * (*su[q])[m];
      aa[q][m] = aa[q][m] * (dl * dl);
      bb[q][m] = bb[q][m] * ((2.0 * dl) * (2.0 * dl));
    }
  }
  // filtered a_ij (parities per direction: src/les_models.f90:681-779)
  const int pa[6][3] = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  vec af[6];
  for (int q = 0; q < 6; ++q) les_fil3(c, aa[q], pa[q][0], pa[q][1], pa[q][2], af[q]);
  vec smagC(N);
  for (size_t m = 0; m < N; ++m) {
    const double mxx = bb[0][m] - af[0][m], myy = bb[1][m] - af[1][m], mzz = bb[2][m] - af[2][m];
    const double mxy = bb[3][m] - af[3][m], mxz = bb[4][m] - af[4][m], myz = bb[5][m] - af[5][m];
    // deviatoric part, statement by statement as the reference writes it
    lxx[m] = lxx[m] - (lxx[m] + lyy[m] + lzz[m]) / 3.0;
    lyy[m] = lyy[m] - (lxx[m] + lyy[m] + lzz[m]) / 3.0;
    lzz[m] = lzz[m] - (lxx[m] + lyy[m] + lzz[m]) / 3.0;
    double v = (lxx[m] * mxx + lyy[m] * myy + lzz[m] * mzz + 2.0 * (lxy[m] * mxy + lxz[m] * mxz + lyz[m] * myz)) /
               (mxx * mxx + myy * myy + mzz * mzz + 2.0 * (mxy * mxy + mxz * mxz + myz * myz));
    if (v > c.maxdsmagcst) v = c.maxdsmagcst;
    if (v < 0.0) v = 0.0;
    smagC[m] = v;
  }
  vec cf;
  les_fil3(c, smagC, 0, 0, 0, cf);
  // mean over z (tools.f90 mean_plane_z), broadcast along z
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  vec cm((size_t)nx * ny, 0.0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      double sum = 0.0;
      for (int k = 0; k < nz; ++k) sum = sum + cf[idx3(i, j, k, nx, ny)];
      cm[(size_t)i + (size_t)nx * j] = sum / (double)nz;
    }
  nut.assign(N, 0.0);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t m = idx3(i, j, k, nx, ny);
        const double dl = c.del[j];
        nut[m] = cm[(size_t)i + (size_t)nx * j] * (dl * dl) * std::sqrt(2.0 * S.srt[m]);
      }
}

// sgs_mom_nonconservative (src/les_models.f90:1091-1250), no IBM.
static void les_sgs(const OxCtx& c, const vec& ux, const vec& uy, const vec& uz, const vec& nut, const StrainT& S,
                    vec& gx, vec& gy, vec& gz) {
  const size_t N = ux.size();
  const int dims[3] = {c.nx, c.ny, c.nz};
  const double* ppy = (c.istret != 0) ? c.ppy.data() : nullptr;
  vec ta(N), td(N), te(N), tf(N), tj(N);
  gx.assign(N, 0.0); gy.assign(N, 0.0); gz.assign(N, 0.0);
  apply3d(c, 0, OP_DER1, 1, nut.data(), ta.data(), dims, nullptr);
  apply3d(c, 0, OP_DER2, 0, ux.data(), td.data(), dims, nullptr);
  apply3d(c, 0, OP_DER2, 1, uy.data(), te.data(), dims, nullptr);
  apply3d(c, 0, OP_DER2, 1, uz.data(), tf.data(), dims, nullptr);
  for (size_t m = 0; m < N; ++m) {
    gx[m] = td[m] * nut[m] + 2.0 * S.sxx[m] * ta[m];
    gy[m] = te[m] * nut[m] + 2.0 * S.sxy[m] * ta[m];
    gz[m] = tf[m] * nut[m] + 2.0 * S.sxz[m] * ta[m];
  }
  apply3d(c, 1, OP_DER1, 1, nut.data(), ta.data(), dims, ppy);
  const vec* us[3] = {&ux, &uy, &uz};
  vec* ts[3] = {&td, &te, &tf};
  const int par[3] = {1, 0, 1};
  for (int q = 0; q < 3; ++q) {
    apply3d(c, 1, OP_DER2, par[q], us[q]->data(), ts[q]->data(), dims, nullptr);
    if (c.istret != 0) {
      apply3d(c, 1, OP_DER1, par[q], us[q]->data(), tj.data(), dims, c.ppy.data());
      vec& t = *ts[q];
      for (size_t m = 0; m < N; ++m) {
        const int j = jrow(m, c.nx, c.ny);
        t[m] = t[m] * c.pp2y[j] - c.pp4y[j] * tj[m];
      }
    }
  }
  for (size_t m = 0; m < N; ++m) {
    gx[m] = gx[m] + nut[m] * td[m] + 2.0 * S.sxy[m] * ta[m];
    gy[m] = gy[m] + nut[m] * te[m] + 2.0 * S.syy[m] * ta[m];
    gz[m] = gz[m] + nut[m] * tf[m] + 2.0 * S.syz[m] * ta[m];
  }
  apply3d(c, 2, OP_DER1, 1, nut.data(), ta.data(), dims, nullptr);
  apply3d(c, 2, OP_DER2, 1, ux.data(), td.data(), dims, nullptr);
  apply3d(c, 2, OP_DER2, 1, uy.data(), te.data(), dims, nullptr);
  apply3d(c, 2, OP_DER2, 0, uz.data(), tf.data(), dims, nullptr);
  for (size_t m = 0; m < N; ++m) {
    gx[m] = gx[m] + nut[m] * td[m] + 2.0 * S.sxz[m] * ta[m];
    gy[m] = gy[m] + nut[m] * te[m] + 2.0 * S.syz[m] * ta[m];
    gz[m] = gz[m] + nut[m] * tf[m] + 2.0 * S.szz[m] * ta[m];
  }
}

// compute_SGS (src/les_models.f90:96-165), iconserv = 0: eddy viscosity and
// the SGS force.
static void les_compute(const OxCtx& c, const vec& ux, const vec& uy, const vec& uz, vec& nut, vec& gx, vec& gy,
                        vec& gz) {
  StrainT S;
  if (c.jles == 1) {
    les_strain(c, ux, uy, uz, S);
    les_smag(c, S, nut);
  } else {
    les_dynsmag(c, ux, uy, uz, nut, S);
  }
  les_sgs(c, ux, uy, uz, nut, S, gx, gy, gz);
}

// ---------------------------------------------------------------------------
// Incompressible step for the plain periodic case
// ---------------------------------------------------------------------------
struct Fields {
  size_t N;
  vec ux, uy, uz;
  vec dux[3], duy[3], duz[3];  // AB history (ntime<=3)
  vec pp3, px, py, pz;
};

// momentum_rhs_eq for the incompressible path without LES or forcing:
// src/transeq.f90:73-591 (skew-symmetric convection + nu*laplacian).
static void momentum_rhs(const OxCtx& c, const vec& ux, const vec& uy, const vec& uz, double xnu, vec& hx, vec& hy,
                         vec& hz) {
  const size_t N = ux.size();
  const int dims[3] = {c.nx, c.ny, c.nz};
  vec ta(N), tb(N), tc(N), td(N), te(N), tf(N), tg(N), th(N), ti(N);
  const double* pp = nullptr;
  // X
  for (size_t m = 0; m < N; ++m) { ta[m] = ux[m] * ux[m]; tb[m] = ux[m] * uy[m]; tc[m] = ux[m] * uz[m]; }
  apply3d(c, 0, OP_DER1, 1, ta.data(), td.data(), dims, nullptr);
  apply3d(c, 0, OP_DER1, 0, tb.data(), te.data(), dims, nullptr);
  apply3d(c, 0, OP_DER1, 0, tc.data(), tf.data(), dims, nullptr);
  apply3d(c, 0, OP_DER1, 0, ux.data(), ta.data(), dims, nullptr);
  apply3d(c, 0, OP_DER1, 1, uy.data(), tb.data(), dims, nullptr);
  apply3d(c, 0, OP_DER1, 1, uz.data(), tc.data(), dims, nullptr);
  vec tg1(N), th1(N), ti1(N);
  for (size_t m = 0; m < N; ++m) {
    tg1[m] = td[m] + ux[m] * ta[m];
    th1[m] = te[m] + ux[m] * tb[m];
    ti1[m] = tf[m] + ux[m] * tc[m];
  }
  // Y
  vec td2(N), te2(N), tf2(N), tg2(N), th2(N), ti2(N);
  for (size_t m = 0; m < N; ++m) { td2[m] = ux[m] * uy[m]; te2[m] = uy[m] * uy[m]; tf2[m] = uz[m] * uy[m]; }
  pp = (c.istret != 0) ? c.ppy.data() : nullptr;  // dery multiplies by ppy when istret != 0
  apply3d(c, 1, OP_DER1, 0, td2.data(), tg2.data(), dims, pp);
  apply3d(c, 1, OP_DER1, 1, te2.data(), th2.data(), dims, pp);
  apply3d(c, 1, OP_DER1, 0, tf2.data(), ti2.data(), dims, pp);
  apply3d(c, 1, OP_DER1, 1, ux.data(), td2.data(), dims, pp);
  apply3d(c, 1, OP_DER1, 0, uy.data(), te2.data(), dims, pp);
  apply3d(c, 1, OP_DER1, 1, uz.data(), tf2.data(), dims, pp);
  for (size_t m = 0; m < N; ++m) {
    tg2[m] = tg2[m] + uy[m] * td2[m];
    th2[m] = th2[m] + uy[m] * te2[m];
    ti2[m] = ti2[m] + uy[m] * tf2[m];
  }
  // Z
  vec td3(N), te3(N), tf3(N), tg3(N), th3(N), ti3(N), ta3(N), tb3(N), tc3(N);
  for (size_t m = 0; m < N; ++m) { td3[m] = ux[m] * uz[m]; te3[m] = uy[m] * uz[m]; tf3[m] = uz[m] * uz[m]; }
  apply3d(c, 2, OP_DER1, 0, td3.data(), tg3.data(), dims, nullptr);
  apply3d(c, 2, OP_DER1, 0, te3.data(), th3.data(), dims, nullptr);
  apply3d(c, 2, OP_DER1, 1, tf3.data(), ti3.data(), dims, nullptr);
  apply3d(c, 2, OP_DER1, 1, ux.data(), td3.data(), dims, nullptr);
  apply3d(c, 2, OP_DER1, 1, uy.data(), te3.data(), dims, nullptr);
  apply3d(c, 2, OP_DER1, 0, uz.data(), tf3.data(), dims, nullptr);
  for (size_t m = 0; m < N; ++m) {
    ta3[m] = tg3[m] + uz[m] * td3[m];
    tb3[m] = th3[m] + uz[m] * te3[m];
    tc3[m] = ti3[m] + uz[m] * tf3[m];
  }
  for (size_t m = 0; m < N; ++m) { td3[m] = ta3[m]; te3[m] = tb3[m]; tf3[m] = tc3[m]; }
  apply3d(c, 2, OP_DER2, 1, ux.data(), ta3.data(), dims, nullptr);
  apply3d(c, 2, OP_DER2, 1, uy.data(), tb3.data(), dims, nullptr);
  apply3d(c, 2, OP_DER2, 0, uz.data(), tc3.data(), dims, nullptr);
  for (size_t m = 0; m < N; ++m) {
    td3[m] = xnu * ta3[m] - 0.5 * td3[m];
    te3[m] = xnu * tb3[m] - 0.5 * te3[m];
    tf3[m] = xnu * tc3[m] - 0.5 * tf3[m];
  }
  // back to Y
  for (size_t m = 0; m < N; ++m) {
    tg2[m] = td3[m] - 0.5 * tg2[m];
    th2[m] = te3[m] - 0.5 * th2[m];
    ti2[m] = tf3[m] - 0.5 * ti2[m];
  }
  apply3d(c, 1, OP_DER2, 1, ux.data(), td2.data(), dims, nullptr);
  apply3d(c, 1, OP_DER2, 0, uy.data(), te2.data(), dims, nullptr);
  apply3d(c, 1, OP_DER2, 1, uz.data(), tf2.data(), dims, nullptr);
  if (c.istret != 0) {
    // stretched mesh: d2/dy2 = deryy*pp2y - pp4y*dery (src/transeq.f90:335-370)
    vec tj(N);
    const vec* us[3] = {&ux, &uy, &uz};
    vec* ts[3] = {&td2, &te2, &tf2};
    const int par[3] = {1, 0, 1};
    for (int q = 0; q < 3; ++q) {
      apply3d(c, 1, OP_DER1, par[q], us[q]->data(), tj.data(), dims, c.ppy.data());
      vec& t = *ts[q];
      for (int k = 0; k < c.nz; ++k)
        for (int j = 0; j < c.ny; ++j)
          for (int i = 0; i < c.nx; ++i) {
            const size_t m = idx3(i, j, k, c.nx, c.ny);
            t[m] = t[m] * c.pp2y[j] - c.pp4y[j] * tj[m];
          }
    }
  }
  vec ta2(N), tb2(N), tc2(N);
  for (size_t m = 0; m < N; ++m) {
    ta2[m] = xnu * td2[m] + tg2[m];
    tb2[m] = xnu * te2[m] + th2[m];
    tc2[m] = xnu * tf2[m] + ti2[m];
  }
  // back to X
  apply3d(c, 0, OP_DER2, 0, ux.data(), td.data(), dims, nullptr);
  apply3d(c, 0, OP_DER2, 1, uy.data(), te.data(), dims, nullptr);
  apply3d(c, 0, OP_DER2, 1, uz.data(), tf.data(), dims, nullptr);
  for (size_t m = 0; m < N; ++m) {
    td[m] = xnu * td[m];
    te[m] = xnu * te[m];
    tf[m] = xnu * tf[m];
  }
  for (size_t m = 0; m < N; ++m) {
    hx[m] = ta2[m] - 0.5 * tg1[m] + td[m];
    hy[m] = tb2[m] - 0.5 * th1[m] + te[m];
    hz[m] = tc2[m] - 0.5 * ti1[m] + tf[m];
  }
  if (c.jles == 1 || c.jles == 3) {
    // src/transeq.f90:475-480: dux1 += sgsx1, ...
    vec nut, gx, gy, gz;
    les_compute(c, ux, uy, uz, nut, gx, gy, gz);
    for (size_t m = 0; m < N; ++m) {
      hx[m] = hx[m] + gx[m];
      hy[m] = hy[m] + gy[m];
      hz[m] = hz[m] + gz[m];
    }
  }
}

// divergence (nlock=1, no IBM): src/navier.f90:257-372; deryvp takes ppyi
// on a stretched mesh.
static void divergence(const OxCtx& c, const vec& ux, const vec& uy, const vec& uz, vec& pp3) {
  const size_t N = ux.size();
  const int dims[3] = {c.nx, c.ny, c.nz};
  const int nxm = c.ax[0].nm, nym = c.ax[1].nm;
  vec pp1((size_t)nxm * c.ny * c.nz), pgy1(pp1.size()), pgz1(pp1.size());
  apply3d(c, 0, OP_DVP, 0, ux.data(), pp1.data(), dims, nullptr);
  apply3d(c, 0, OP_IVP, 1, uy.data(), pgy1.data(), dims, nullptr);
  apply3d(c, 0, OP_IVP, 1, uz.data(), pgz1.data(), dims, nullptr);
  const int d2[3] = {nxm, c.ny, c.nz};
  vec upi2((size_t)nxm * nym * c.nz), duydypi2(upi2.size());
  apply3d(c, 1, OP_IVP, 1, pp1.data(), upi2.data(), d2, nullptr);
  apply3d(c, 1, OP_DVP, 0, pgy1.data(), duydypi2.data(), d2, c.istret != 0 ? c.ppyi.data() : nullptr);
  for (size_t m = 0; m < upi2.size(); ++m) duydypi2[m] = duydypi2[m] + upi2[m];
  apply3d(c, 1, OP_IVP, 1, pgz1.data(), upi2.data(), d2, nullptr);
  const int d3[3] = {nxm, nym, c.nz};
  const int nzm = c.ax[2].nm;
  pp3.assign((size_t)nxm * nym * nzm, 0.0);
  vec po3(pp3.size());
  apply3d(c, 2, OP_IVP, 1, duydypi2.data(), pp3.data(), d3, nullptr);
  apply3d(c, 2, OP_DVP, 0, upi2.data(), po3.data(), d3, nullptr);
  for (size_t m = 0; m < pp3.size(); ++m) pp3[m] = pp3[m] + po3[m];
  (void)N;
}

// gradp: src/navier.f90:386-432; derypv takes ppy on a stretched mesh.  The
// wall-gradient storage of src/navier.f90:434-499 is done by the caller.
static void gradp(const OxCtx& c, const vec& pp3, vec& px, vec& py, vec& pz) {
  const int nxm = c.ax[0].nm, nym = c.ax[1].nm, nzm = c.ax[2].nm;
  const int d3[3] = {nxm, nym, nzm};
  vec ppi3((size_t)nxm * nym * c.nz), pgz3(ppi3.size());
  apply3d(c, 2, OP_IPV, 1, pp3.data(), ppi3.data(), d3, nullptr);
  apply3d(c, 2, OP_DPV, 1, pp3.data(), pgz3.data(), d3, nullptr);
  const int d2[3] = {nxm, nym, c.nz};
  vec ppi2((size_t)nxm * c.ny * c.nz), pgy2(ppi2.size()), pgzi2(ppi2.size());
  apply3d(c, 1, OP_IPV, 1, ppi3.data(), ppi2.data(), d2, nullptr);
  apply3d(c, 1, OP_DPV, 1, ppi3.data(), pgy2.data(), d2, c.istret != 0 ? c.ppy.data() : nullptr);
  apply3d(c, 1, OP_IPV, 1, pgz3.data(), pgzi2.data(), d2, nullptr);
  const int d1[3] = {nxm, c.ny, c.nz};
  apply3d(c, 0, OP_DPV, 1, ppi2.data(), px.data(), d1, nullptr);
  apply3d(c, 0, OP_IPV, 1, pgy2.data(), py.data(), d1, nullptr);
  apply3d(c, 0, OP_IPV, 1, pgzi2.data(), pz.data(), d1, nullptr);
}

// ---------------------------------------------------------------------------
// C interface used by the tests (ctypes)
// ---------------------------------------------------------------------------
extern "C" {

// ivals: nx,ny,nz, nclx1,nclxn, ncly1,nclyn, nclz1,nclzn, ifirstder,isecondder,ipinter, istret
// dvals: xlx,yly,zlz, filter_alpha, nu0nu, cnu, beta
void* ox_create(const int* iv, const double* dv) {
  OxCtx* c = new OxCtx();
  c->nx = iv[0]; c->ny = iv[1]; c->nz = iv[2];
  c->opts.ifirstder = iv[9]; c->opts.isecondder = iv[10]; c->opts.ipinter = iv[11];
  c->xlx = dv[0]; c->yly = dv[1]; c->zlz = dv[2];
  c->opts.filter_alpha = dv[3]; c->opts.nu0nu = dv[4]; c->opts.cnu = dv[5];
  setup_axis(c->ax[0], c->nx, c->xlx, iv[3], iv[4], c->opts);
  setup_axis(c->ax[1], c->ny, c->yly, iv[5], iv[6], c->opts);
  setup_axis(c->ax[2], c->nz, c->zlz, iv[7], iv[8], c->opts);
  c->istret = iv[12];
  c->beta = dv[6];
  stretching_setup(*c);
  if (c->ax[0].periodic && !c->ax[1].periodic && c->ax[2].periodic) {
    vec tmp;
    waves_axis(c->ax[0], c->kx2, c->trx10);
    waves_axis(c->ax[2], c->kz2, c->trz10);
    waves_y010(*c, c->yky10, c->yk210, c->eys10, c->try10);
    abxyz_axis(c->nx, c->sax, c->sbx);
    abxyz_half(c->ax[1].nm, c->say, c->sby);
    abxyz_axis(c->nz, c->saz, c->sbz);
  }
  if (c->ax[0].periodic && c->ax[1].periodic && c->ax[2].periodic) {
    waves_axis(c->ax[0], c->kx2, c->tx);
    waves_axis(c->ax[1], c->ky2, c->ty);
    waves_axis(c->ax[2], c->kz2, c->tz);
    abxyz_axis(c->nx, c->sax, c->sbx);
    abxyz_axis(c->ny, c->say, c->sby);
    abxyz_axis(c->nz, c->saz, c->sbz);
  }
  return c;
}

void ox_destroy(void* h) { delete (OxCtx*)h; }

int ox_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// Apply one operator.  dims = input dims (nx_in, ny_in, nz_in); pp may be NULL.
int ox_op(void* h, int axis, int op, int npaire, const double* u, double* t, const int* dims, const double* pp) {
  const OxCtx* c = (const OxCtx*)h;
  if (axis < 0 || axis > 2 || op < 0 || op > 6) return -1;
  int d[3] = {dims[0], dims[1], dims[2]};
  apply3d(*c, axis, op, npaire, u, t, d, pp);
  return 0;
}

// Coefficient vectors, for the tests.  which: 0..5 = ff,fs,fw,ffp,fsp,fwp;
// 6..11 = sf,ss,sw,sfp,ssp,swp; 12..17 = fiff,fifs,fifw,fiffp,fifsp,fifwp;
// 18..20 = cf6,cs6,cw6; 21..23 = cif6,cis6,ciw6; 24..26 = cifp6,cisp6,ciwp6;
// 27..29 = cfip6,csip6,cwip6; 30..32 = cifip6,cisip6,ciwip6;
// 33 = modified wavenumber^2 table; 34 = interpolation transfer table.
int ox_coeffs(void* h, int axis, int which, double* out) {
  const OxCtx* c = (const OxCtx*)h;
  const Axis& a = c->ax[axis];
  const vec* tab[] = {&a.ff, &a.fs, &a.fw, &a.ffp, &a.fsp, &a.fwp, &a.sf, &a.ss, &a.sw, &a.sfp, &a.ssp, &a.swp,
                      &a.fiff, &a.fifs, &a.fifw, &a.fiffp, &a.fifsp, &a.fifwp, &a.cf6, &a.cs6, &a.cw6,
                      &a.cif6, &a.cis6, &a.ciw6, &a.cifp6, &a.cisp6, &a.ciwp6, &a.cfip6, &a.csip6, &a.cwip6,
                      &a.cifip6, &a.cisip6, &a.ciwip6};
  const vec* v = nullptr;
  if (which >= 0 && which < 33) v = tab[which];
  else if (which == 33) v = axis == 0 ? &c->kx2 : axis == 1 ? &c->ky2 : &c->kz2;
  else if (which == 34) v = axis == 0 ? &c->tx : axis == 1 ? &c->ty : &c->tz;
  if (!v) return -1;
  std::memcpy(out, v->data(), v->size() * sizeof(double));
  return (int)v->size();
}

// Scalar coefficients of an axis, in a fixed order (for the tests).
int ox_scalars(void* h, int axis, double* out) {
  const Axis& a = ((const OxCtx*)h)->ax[axis];
  const double v[] = {a.alfai, a.afi, a.bfi, a.alsai, a.asi, a.bsi, a.csi, a.dsi, a.fiali, a.fiai, a.fibi, a.fici,
                      a.fidi, a.alcai6, a.aci6, a.bci6, a.ailcai6, a.aici6, a.bici6, a.cicoef6, a.dici6, a.d};
  const int n = sizeof(v) / sizeof(v[0]);
  for (int i = 0; i < n; ++i) out[i] = v[i];
  return n;
}

// ---------------------------------------------------------------------------
// Poisson solve with free-slip x and y (and z free-slip or periodic):
// src/poisson.f90:1019-1465 (poisson_11x, istret = 0).  The p-mesh sizes
// NX = nxm, NY = nym, NZ = nzm (nz if z is periodic); spectral array
// (NX, NY, NZ/2+1) as 2DECOMP's PHYSICAL_IN_Z transform leaves it.
// ---------------------------------------------------------------------------

// Wavenumber^2 and interpolation transfer of the modes of a free-slip axis
// (waves, bcx = 1 / bcy = 1: src/poisson.f90:1588-1601, 1621-1637; the
// transfer of :1740-1760), m = 0..nm-1.
void waves_slip(const Axis& a, vec& k2, vec& tr) {
  const int nm = a.nm;
  k2.assign(nm, 0.0);
  tr.assign(nm, 0.0);
  vec es(nm, 0.0);
  for (int i = 1; i <= nm; ++i) {
    const double w = TWOPI * 0.5 * (double)(i - 1) / (double)nm;
    double wp = a.aci6 * 2.0 * a.d * std::sin(w * 0.5) + (a.bci6 * 2.0 * a.d) * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * a.alcai6 * std::cos(w));
    const double t = (double)nm * wp / a.len;
    k2[i - 1] = t * t;
    es[i - 1] = (double)nm * w / a.len;
  }
  k2[0] = 0.0;
  es[0] = 0.0;
  for (int i = 0; i < nm; ++i) tr[i] = transfer(a, es[i] * a.d);
}

// kxyz of poisson_11x (src/poisson.f90:1725-1806): (re, im) per spectral point
// (i, j, k), i fastest, k < NZ/2+1.  For a periodic z both parts are equal.
void kxyz_11x(const OxCtx& c, vec& kre, vec& kim) {
  const Axis &ax = c.ax[0], &ay = c.ax[1], &az = c.ax[2];
  const int NX = ax.nm, NY = ay.nm, NZ = az.nm, NZ2 = NZ / 2 + 1;
  vec kx2, trx, ky2, try_;
  waves_slip(ax, kx2, trx);
  waves_slip(ay, ky2, try_);
  kre.assign((size_t)NX * NY * NZ2, 0.0);
  kim.assign(kre.size(), 0.0);
  if (az.periodic) {
    vec kz2, trz;
    waves_axis(az, kz2, trz);
    for (int k = 0; k < NZ2; ++k)
      for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i) {
          const double txz = try_[j] * trz[k], tyz = trx[i] * trz[k], txy = trx[i] * try_[j];
          const double xt2 = kx2[i] * (txz * txz), yt2 = ky2[j] * (tyz * tyz), zt2 = kz2[k] * (txy * txy);
          const size_t q = (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k);
          kre[q] = xt2 + yt2 + zt2;
          kim[q] = kre[q];
        }
    return;
  }
  // free-slip z: the real part carries mode k, the imaginary part mode NZ-k
  for (int k = 1; k <= NZ2; ++k) {
    const double w = PI * (double)(k - 1) / (double)NZ;
    const double w1 = PI * (double)(NZ - k + 1) / (double)NZ;
    double wp = az.aci6 * 2.0 * az.d * std::sin(w * 0.5) + (az.bci6 * 2.0 * az.d) * std::sin(3.0 * 0.5 * w);
    wp = wp / (1.0 + 2.0 * az.alcai6 * std::cos(w));
    double w1p = az.aci6 * 2.0 * az.d * std::sin(w1 * 0.5) + (az.bci6 * 2.0 * az.d) * std::sin(3.0 * 0.5 * w1);
    w1p = w1p / (1.0 + 2.0 * az.alcai6 * std::cos(w1));
    const double kzr = (double)NZ * wp / az.len, kzi = (double)NZ * w1p / az.len;
    const double zk2r = kzr * kzr, zk2i = kzi * kzi;
    const double rlezs = ((double)NZ * w / az.len) * az.d, iyezs = ((double)NZ * w1 / az.len) * az.d;
    const double ztr = 2.0 * (az.bici6 * std::cos(rlezs * 1.5) + az.cicoef6 * std::cos(rlezs * 2.5) +
                              az.dici6 * std::cos(rlezs * 3.5));
    const double zti = 2.0 * (az.bici6 * std::cos(iyezs * 1.5) + az.cicoef6 * std::cos(iyezs * 2.5) +
                              az.dici6 * std::cos(iyezs * 3.5));
    const double zt1r = 2.0 * az.aici6 * std::cos(rlezs * 0.5), zt1i = 2.0 * az.aici6 * std::cos(iyezs * 0.5);
    const double z1r = 1.0 + 2.0 * az.ailcai6 * std::cos(rlezs), z1i = 1.0 + 2.0 * az.ailcai6 * std::cos(iyezs);
    const double t1r = (zt1r + ztr) / z1r, t1i = (zt1i + zti) / z1i;
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i) {
        const double t2 = try_[j], t3 = trx[i];
        const double t4r = t2 * t2 * (t1r * t1r), t4i = t2 * t2 * (t1i * t1i);
        const double t5r = t3 * t3 * (t1r * t1r), t5i = t3 * t3 * (t1i * t1i);
        const double t6 = (t3 * t2) * (t3 * t2);
        const size_t q = (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * (k - 1));
        kre[q] = t4r * kx2[i] + t5r * ky2[j] + t6 * zk2r;
        kim[q] = t4i * kx2[i] + t5i * ky2[j] + t6 * zk2i;
      }
  }
}

// even / odd reorder of one axis (src/poisson.f90:1041-1098): v[d] = u[p(d)]
inline int slip_perm(int d, int n) { return (d < n / 2) ? 2 * d : 2 * n - 2 * d - 1; }

static void poisson_11x(const OxCtx& c, double* rhs) {
  const int NX = c.ax[0].nm, NY = c.ax[1].nm, NZ = c.ax[2].nm, NZ2 = NZ / 2 + 1;
  const bool bcz = !c.ax[2].periodic;
  const size_t N = (size_t)NX * NY * NZ;
  {
    vec t(rhs, rhs + N);
    for (int k = 0; k < NZ; ++k)
      for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i)
          rhs[idx3(i, j, k, NX, NY)] =
              t[idx3(slip_perm(i, NX), slip_perm(j, NY), bcz ? slip_perm(k, NZ) : k, NX, NY)];
  }
  std::vector<cplx> cw((size_t)NX * NY * NZ2);
  auto CW = [&](int i, int j, int k) -> cplx& { return cw[(size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k)]; };
#pragma omp parallel
  {
    std::vector<cplx> line, work;
#pragma omp for collapse(2)
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i) {
        line.assign(NZ, cplx(0, 0));
        for (int k = 0; k < NZ; ++k) line[k] = cplx(rhs[idx3(i, j, k, NX, NY)], 0.0);
        fft1d(line.data(), NZ, -1, work);
        for (int k = 0; k < NZ2; ++k) CW(i, j, k) = line[k];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < NZ2; ++k)
      for (int i = 0; i < NX; ++i) {
        line.resize(NY);
        for (int j = 0; j < NY; ++j) line[j] = CW(i, j, k);
        fft1d(line.data(), NY, -1, work);
        for (int j = 0; j < NY; ++j) CW(i, j, k) = line[j];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < NZ2; ++k)
      for (int j = 0; j < NY; ++j) {
        line.resize(NX);
        for (int i = 0; i < NX; ++i) line[i] = CW(i, j, k);
        fft1d(line.data(), NX, -1, work);
        for (int i = 0; i < NX; ++i) CW(i, j, k) = line[i];
      }
  }
  for (auto& v : cw) v = cplx(v.real() / (double)NX / (double)NY / (double)NZ, v.imag() / (double)NX / (double)NY / (double)NZ);
  vec sax, sbx, say, sby, saz, sbz;
  abxyz_half(NX, sax, sbx);
  abxyz_half(NY, say, sby);
  if (bcz) abxyz_half(NZ, saz, sbz);
  else abxyz_axis(NZ, saz, sbz);
  // post-processing in z, y, x (src/poisson.f90:1117-1198)
  for (int k = 0; k < NZ2; ++k)
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i) {
        cplx& v = CW(i, j, k);
        const double t1 = v.real(), t2 = v.imag();
        v = cplx(t1 * sbz[k] + t2 * saz[k], t2 * sbz[k] - t1 * saz[k]);
      }
  auto pair_fwd = [](cplx a, cplx b, double bb, double aa) {
    const double t1 = a.real(), t2 = a.imag(), t3 = b.real(), t4 = b.imag();
    const double x1 = t1 * bb * 0.5, x2 = t1 * aa * 0.5, x3 = t2 * bb * 0.5, x4 = t2 * aa * 0.5;
    const double x5 = t3 * bb * 0.5, x6 = t3 * aa * 0.5, x7 = t4 * bb * 0.5, x8 = t4 * aa * 0.5;
    return cplx(x1 + x4 + x5 - x8, -x2 + x3 + x6 + x7);
  };
  auto pair_bwd = [](cplx a, cplx b, double bb, double aa) {
    const double t1 = a.real(), t2 = a.imag(), t3 = b.real(), t4 = b.imag();
    const double x1 = t1 * bb, x2 = t1 * aa, x3 = t2 * bb, x4 = t2 * aa;
    const double x5 = t3 * bb, x6 = t3 * aa, x7 = t4 * bb, x8 = t4 * aa;
    return cplx(x1 - x4 + x6 + x7, -(-x2 - x3 + x5 - x8));
  };
  std::vector<cplx> cb(cw.size());
  auto CB = [&](int i, int j, int k) -> cplx& { return cb[(size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k)]; };
  for (int k = 0; k < NZ2; ++k)
    for (int i = 0; i < NX; ++i) {
      CB(i, 0, k) = CW(i, 0, k);
      for (int j = 1; j < NY; ++j) CB(i, j, k) = pair_fwd(CW(i, j, k), CW(i, NY - j, k), sby[j], say[j]);
    }
  for (int k = 0; k < NZ2; ++k)
    for (int j = 0; j < NY; ++j) {
      CW(0, j, k) = CB(0, j, k);
      for (int i = 1; i < NX; ++i) CW(i, j, k) = pair_fwd(CB(i, j, k), CB(NX - i, j, k), sbx[i], sax[i]);
    }
  // division (src/poisson.f90:1200-1228)
  vec kre, kim;
  kxyz_11x(c, kre, kim);
  const double eps = 1.0e-16;
  for (size_t q = 0; q < cw.size(); ++q) {
    const double t1 = kre[q], t2 = kim[q];
    cplx& v = cw[q];
    if (std::fabs(t1) < eps && std::fabs(t2) < eps) v = cplx(0.0, 0.0);
    if (std::fabs(t1) < eps && std::fabs(t2) >= eps) v = cplx(0.0, v.imag() / (-t2));
    if (std::fabs(t1) >= eps && std::fabs(t2) < eps) v = cplx(v.real() / (-t1), 0.0);
    if (std::fabs(t1) >= eps && std::fabs(t2) >= eps) v = cplx(v.real() / (-t1), v.imag() / (-t2));
  }
  // backward post-processing in x, y, z (src/poisson.f90:1337-1411)
  for (int k = 0; k < NZ2; ++k)
    for (int j = 0; j < NY; ++j) {
      CB(0, j, k) = CW(0, j, k);
      for (int i = 1; i < NX; ++i) CB(i, j, k) = pair_bwd(CW(i, j, k), CW(NX - i, j, k), sbx[i], sax[i]);
    }
  for (int k = 0; k < NZ2; ++k)
    for (int i = 0; i < NX; ++i) {
      CW(i, 0, k) = CB(i, 0, k);
      for (int j = 1; j < NY; ++j) CW(i, j, k) = pair_bwd(CB(i, j, k), CB(i, NY - j, k), sby[j], say[j]);
    }
  for (int k = 0; k < NZ2; ++k)
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i) {
        cplx& v = CW(i, j, k);
        const double t1 = v.real(), t2 = v.imag();
        v = cplx(t1 * sbz[k] - t2 * saz[k], t2 * sbz[k] + t1 * saz[k]);
      }
  // c2r (x, y inverse, then z complex-to-real), then the inverse reorders
  vec out(N);
#pragma omp parallel
  {
    std::vector<cplx> line, work;
#pragma omp for collapse(2)
    for (int k = 0; k < NZ2; ++k)
      for (int j = 0; j < NY; ++j) {
        line.resize(NX);
        for (int i = 0; i < NX; ++i) line[i] = CW(i, j, k);
        fft1d(line.data(), NX, +1, work);
        for (int i = 0; i < NX; ++i) CW(i, j, k) = line[i];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < NZ2; ++k)
      for (int i = 0; i < NX; ++i) {
        line.resize(NY);
        for (int j = 0; j < NY; ++j) line[j] = CW(i, j, k);
        fft1d(line.data(), NY, +1, work);
        for (int j = 0; j < NY; ++j) CW(i, j, k) = line[j];
      }
#pragma omp for collapse(2)
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i) {
        line.assign(NZ, cplx(0, 0));
        for (int k = 0; k < NZ2; ++k) line[k] = CW(i, j, k);
        for (int k = NZ2; k < NZ; ++k) line[k] = std::conj(CW(i, j, NZ - k));
        line[0] = cplx(line[0].real(), 0.0);
        if (NZ % 2 == 0) line[NZ / 2] = cplx(line[NZ / 2].real(), 0.0);
        fft1d(line.data(), NZ, +1, work);
        for (int k = 0; k < NZ; ++k) out[idx3(i, j, k, NX, NY)] = line[k].real();
      }
  }
  for (int k = 0; k < NZ; ++k)
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i)
        rhs[idx3(slip_perm(i, NX), slip_perm(j, NY), bcz ? slip_perm(k, NZ) : k, NX, NY)] = out[idx3(i, j, k, NX, NY)];
}

int ox_poisson(void* h, double* rhs) {
  const OxCtx* c = (const OxCtx*)h;
  if (c->ax[0].periodic && c->ax[1].periodic && c->ax[2].periodic) {
    poisson_000(*c, rhs);
    return 0;
  }
  if (c->ax[0].periodic && !c->ax[1].periodic && c->ax[2].periodic) {
    if (c->istret == 3) return -2;
    poisson_010(*c, rhs);
    return 0;
  }
  if (slip_axis(c->ax[0]) && slip_axis(c->ax[1]) && (c->ax[2].periodic || slip_axis(c->ax[2]))) {
    if (c->istret != 0) return -2;
    poisson_11x(*c, rhs);
    return 0;
  }
  return -2;
}

// Explicit LES model for the right-hand side (src/les_models.f90):
// jles 0 none, 1 Smagorinsky, 3 dynamic Smagorinsky.  Sets the filter width
// del(j) of init_explicit_les (src/les_models.f90:27-30) and the alpha = 0
// filter dynsmag uses (filter(zero), src/les_models.f90:393).
int ox_set_les(void* h, int jles, double smagcst, double maxdsmagcst) {
  OxCtx* c = (OxCtx*)h;
  if (jles != 0 && jles != 1 && jles != 3) return -1;
  c->jles = jles;
  c->smagcst = smagcst;
  c->maxdsmagcst = maxdsmagcst;
  const int ny = c->ny;
  c->del.assign(ny, 0.0);
  for (int j = 0; j < ny - 1; ++j)
    c->del[j] = std::pow(c->ax[0].d * (c->yp[j + 1] - c->yp[j]) * c->ax[2].d, 1.0 / 3.0);
  c->del[ny - 1] = c->del[ny - 2];
  for (int a = 0; a < 3; ++a) {
    c->axf[a] = c->ax[a];
    filter_coefficients(c->axf[a], 0.0);
  }
  return 0;
}

// Eddy viscosity and SGS force of compute_SGS for the current LES model.
int ox_les(void* h, const double* ux, const double* uy, const double* uz, double* nut, double* gx, double* gy,
           double* gz) {
  const OxCtx* c = (const OxCtx*)h;
  if (c->jles != 1 && c->jles != 3) return -1;
  const size_t N = (size_t)c->nx * c->ny * c->nz;
  vec a(ux, ux + N), b(uy, uy + N), d(uz, uz + N), n, x, y, z;
  les_compute(*c, a, b, d, n, x, y, z);
  std::memcpy(nut, n.data(), N * sizeof(double));
  std::memcpy(gx, x.data(), N * sizeof(double));
  std::memcpy(gy, y.data(), N * sizeof(double));
  std::memcpy(gz, z.data(), N * sizeof(double));
  return 0;
}

// Stretching metrics: which = 0..7 -> yp, ypi, ppy, pp2y, pp4y, ppyi, pp2yi,
// pp4yi; 8 -> {alpha}.
int ox_stretching(void* h, int which, double* out) {
  const OxCtx* c = (const OxCtx*)h;
  const vec* tab[] = {&c->yp, &c->ypi, &c->ppy, &c->pp2y, &c->pp4y, &c->ppyi, &c->pp2yi, &c->pp4yi};
  if (which == 8) { out[0] = c->alpha; return 1; }
  if (which < 0 || which > 7) return -1;
  std::memcpy(out, tab[which]->data(), tab[which]->size() * sizeof(double));
  return (int)tab[which]->size();
}

int ox_divergence(void* h, const double* ux, const double* uy, const double* uz, double* pp3) {
  const OxCtx* c = (const OxCtx*)h;
  const size_t N = (size_t)c->nx * c->ny * c->nz;
  vec a(ux, ux + N), b(uy, uy + N), d(uz, uz + N), p;
  divergence(*c, a, b, d, p);
  std::memcpy(pp3, p.data(), p.size() * sizeof(double));
  return 0;
}

int ox_gradp(void* h, const double* pp3, double* px, double* py, double* pz) {
  const OxCtx* c = (const OxCtx*)h;
  const size_t N = (size_t)c->nx * c->ny * c->nz;
  const size_t M = (size_t)c->ax[0].nm * c->ax[1].nm * c->ax[2].nm;
  vec p(pp3, pp3 + M), a(N), b(N), d(N);
  gradp(*c, p, a, b, d);
  std::memcpy(px, a.data(), N * sizeof(double));
  std::memcpy(py, b.data(), N * sizeof(double));
  std::memcpy(pz, d.data(), N * sizeof(double));
  return 0;
}

int ox_rhs(void* h, const double* ux, const double* uy, const double* uz, double xnu, double* hx, double* hy,
           double* hz) {
  const OxCtx* c = (const OxCtx*)h;
  const size_t N = (size_t)c->nx * c->ny * c->nz;
  vec a(ux, ux + N), b(uy, uy + N), d(uz, uz + N), x(N), y(N), z(N);
  momentum_rhs(*c, a, b, d, xnu, x, y, z);
  std::memcpy(hx, x.data(), N * sizeof(double));
  std::memcpy(hy, y.data(), N * sizeof(double));
  std::memcpy(hz, z.data(), N * sizeof(double));
  return 0;
}

// TGV statistics of src/Case-TGV.f90:189-477 (postprocess_tgv) for the periodic
// box: out = {eek, eps, eps2, enst}.
int ox_tgv_stats(void* h, const double* ux, const double* uy, const double* uz, double xnu, double* out) {
  const OxCtx* c = (const OxCtx*)h;
  const size_t N = (size_t)c->nx * c->ny * c->nz;
  const int dims[3] = {c->nx, c->ny, c->nz};
  vec ta(N), tb(N), tc(N), td(N), te(N), tf(N), tg(N), th(N), ti(N);
  apply3d(*c, 0, OP_DER1, 0, ux, ta.data(), dims, nullptr);
  apply3d(*c, 0, OP_DER1, 1, uy, tb.data(), dims, nullptr);
  apply3d(*c, 0, OP_DER1, 1, uz, tc.data(), dims, nullptr);
  apply3d(*c, 1, OP_DER1, 1, ux, td.data(), dims, nullptr);
  apply3d(*c, 1, OP_DER1, 0, uy, te.data(), dims, nullptr);
  apply3d(*c, 1, OP_DER1, 1, uz, tf.data(), dims, nullptr);
  apply3d(*c, 2, OP_DER1, 1, ux, tg.data(), dims, nullptr);
  apply3d(*c, 2, OP_DER1, 1, uy, th.data(), dims, nullptr);
  apply3d(*c, 2, OP_DER1, 0, uz, ti.data(), dims, nullptr);
  double enst = 0, eps = 0, eek = 0, eps2 = 0;
  // sums over the points the reference visits: the last point of a free-slip
  // axis is left out, and the mean is over nxc*nyc*nzc (nxc = nxm there;
  // src/Case-TGV.f90:211-241)
  const int sx = (c->ax[0].ncl1 == 1) ? c->nx - 1 : c->nx;
  const int sy = (c->ax[1].ncl1 == 1) ? c->ny - 1 : c->ny;
  const int sz = (c->ax[2].ncl1 == 1) ? c->nz - 1 : c->nz;
  const double nc = (double)(c->ax[0].ncl1 == 1 ? c->ax[0].nm : c->nx) * (c->ax[1].ncl1 == 1 ? c->ax[1].nm : c->ny) *
                    (c->ax[2].ncl1 == 1 ? c->ax[2].nm : c->nz);
  auto box = [&](auto f) {
    for (int k = 0; k < sz; ++k)
      for (int j = 0; j < sy; ++j)
        for (int i = 0; i < sx; ++i) f(idx3(i, j, k, c->nx, c->ny));
  };
  box([&](size_t m) {
    const double a1 = tf[m] - th[m], a2 = tg[m] - tc[m], a3 = tb[m] - td[m];
    enst = enst + 0.5 * (a1 * a1 + a2 * a2 + a3 * a3);
  });
  enst = enst / nc;
  box([&](size_t m) {
    const double s1 = 2.0 * ta[m], s2 = 2.0 * te[m], s3 = 2.0 * ti[m];
    const double s4 = td[m] + tb[m], s5 = tg[m] + tc[m], s6 = th[m] + tf[m];
    eps = eps + 0.5 * xnu * (s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4) + 2.0 * (s5 * s5) + 2.0 * (s6 * s6));
  });
  eps = eps / nc;
  box([&](size_t m) { eek = eek + 0.5 * (ux[m] * ux[m] + uy[m] * uy[m] + uz[m] * uz[m]); });
  eek = eek / nc;
  apply3d(*c, 0, OP_DER2, 0, ux, ta.data(), dims, nullptr);
  apply3d(*c, 0, OP_DER2, 1, uy, tb.data(), dims, nullptr);
  apply3d(*c, 0, OP_DER2, 1, uz, tc.data(), dims, nullptr);
  apply3d(*c, 1, OP_DER2, 1, ux, td.data(), dims, nullptr);
  apply3d(*c, 1, OP_DER2, 0, uy, te.data(), dims, nullptr);
  apply3d(*c, 1, OP_DER2, 1, uz, tf.data(), dims, nullptr);
  apply3d(*c, 2, OP_DER2, 1, ux, tg.data(), dims, nullptr);
  apply3d(*c, 2, OP_DER2, 1, uy, th.data(), dims, nullptr);
  apply3d(*c, 2, OP_DER2, 0, uz, ti.data(), dims, nullptr);
  box([&](size_t m) {
    const double di = (-xnu) * (ux[m] * (ta[m] + td[m] + tg[m]) + uy[m] * (tb[m] + te[m] + th[m]) +
                                uz[m] * (tc[m] + tf[m] + ti[m]));
    eps2 = eps2 + di;
  });
  eps2 = eps2 / nc;
  out[0] = eek; out[1] = eps; out[2] = eps2; out[3] = enst;
  return 0;
}

// Run the plain periodic incompressible solver: time loop of
// src/xcompact3d.f90:29-102 with transeq -> intt -> solve_poisson -> cor_vel.
// itimescheme: 3 = AB3 (Euler, AB2 start-up), 5 = RK3.  The velocity arrays are
// advanced in place.  Statistics {t, eek, eps, eps2, enst} are written every
// `every` steps into stats (rows), t = (itime-1)*dt as in the reference's file.
int ox_run(void* h, double* ux_, double* uy_, double* uz_, int nsteps, double dt, double xnu, int itimescheme,
           int every, double* stats, double* divmax) {
  const OxCtx* c = (const OxCtx*)h;
  const size_t N = (size_t)c->nx * c->ny * c->nz;
  vec ux(ux_, ux_ + N), uy(uy_, uy_ + N), uz(uz_, uz_ + N);
  const int ntime = (itimescheme == 3) ? 3 : 2;
  std::vector<vec> dux(ntime, vec(N, 0.0)), duy(ntime, vec(N, 0.0)), duz(ntime, vec(N, 0.0));
  double adt[3] = {0, 0, 0}, bdt[3] = {0, 0, 0}, cdt[3] = {0, 0, 0}, gdt[3] = {0, 0, 0};
  int nsub = 1;
  if (itimescheme == 3) {  // src/variables.f90:1366-1377
    adt[0] = (23.0 / 12.0) * dt; bdt[0] = -(16.0 / 12.0) * dt; cdt[0] = (5.0 / 12.0) * dt;
    gdt[0] = adt[0] + bdt[0] + cdt[0];
  } else if (itimescheme == 5) {  // src/variables.f90:1389-1400
    nsub = 3;
    adt[0] = (8.0 / 15.0) * dt; bdt[0] = 0; gdt[0] = adt[0];
    adt[1] = (5.0 / 12.0) * dt; bdt[1] = (-17.0 / 60.0) * dt; gdt[1] = adt[1] + bdt[1];
    adt[2] = (3.0 / 4.0) * dt; bdt[2] = (-5.0 / 12.0) * dt; gdt[2] = adt[2] + bdt[2];
  } else {
    return -3;
  }
  vec pp3, px(N), py(N), pz(N);
  int row = 0;
  double dmax = 0;
  for (int itime = 1; itime <= nsteps; ++itime) {
    for (int itr = 1; itr <= nsub; ++itr) {
      momentum_rhs(*c, ux, uy, uz, xnu, dux[0], duy[0], duz[0]);
      // intt: src/time_integrators.f90:18-187
      vec* vars[3] = {&ux, &uy, &uz};
      std::vector<vec>* dvs[3] = {&dux, &duy, &duz};
      for (int q = 0; q < 3; ++q) {
        vec& v = *vars[q];
        std::vector<vec>& d = *dvs[q];
        if (itimescheme == 3) {
          if (itime == 1) {
            for (size_t m = 0; m < N; ++m) v[m] = dt * d[0][m] + v[m];
          } else if (itime == 2) {
            for (size_t m = 0; m < N; ++m) v[m] = 1.5 * dt * d[0][m] - 0.5 * dt * d[1][m] + v[m];
            d[2] = d[1];
          } else {
            for (size_t m = 0; m < N; ++m)
              v[m] = adt[0] * d[0][m] + bdt[0] * d[1][m] + cdt[0] * d[2][m] + v[m];
            d[2] = d[1];
          }
          d[1] = d[0];
        } else {
          if (itr == 1) {
            for (size_t m = 0; m < N; ++m) v[m] = gdt[0] * d[0][m] + v[m];
          } else {
            for (size_t m = 0; m < N; ++m) v[m] = adt[itr - 1] * d[0][m] + bdt[itr - 1] * d[1][m] + v[m];
          }
          d[1] = d[0];
        }
      }
      divergence(*c, ux, uy, uz, pp3);
      if (ox_poisson(h, pp3.data()) != 0) return -2;
      gradp(*c, pp3, px, py, pz);
      for (size_t m = 0; m < N; ++m) { ux[m] = ux[m] - px[m]; uy[m] = uy[m] - py[m]; uz[m] = uz[m] - pz[m]; }
    }
    if (every > 0 && itime % every == 0 && stats) {
      double st[4];
      ox_tgv_stats(h, ux.data(), uy.data(), uz.data(), xnu, st);
      stats[row * 5 + 0] = (itime - 1) * dt;
      for (int q = 0; q < 4; ++q) stats[row * 5 + 1 + q] = st[q];
      ++row;
    }
  }
  if (divmax) {
    vec p;
    divergence(*c, ux, uy, uz, p);
    for (double v : p) dmax = std::max(dmax, std::fabs(v));
    *divmax = dmax;
  }
  std::memcpy(ux_, ux.data(), N * sizeof(double));
  std::memcpy(uy_, uy.data(), N * sizeof(double));
  std::memcpy(uz_, uz.data(), N * sizeof(double));
  return row;
}

// Channel flow time loop (src/xcompact3d.f90:29-102 with the channel case):
// per sub-step boundary_conditions -> channel_cfr (src/Case-Channel.f90:221-264,
// constant flow rate 2/3), momentum_rhs_eq + momentum_forcing_channel
// (src/Case-Channel.f90:392-421, rotation while itime < spinup_time), intt,
// pre_correc's no-slip wall values (src/navier.f90:614-700), divergence,
// poisson_010, gradp with the wall pressure-gradient storage
// (src/navier.f90:456-477) and cor_vel.  Walls at y = 0 and y = Ly
// (ncly1 = nclyn = 2) with zero wall velocity; x and z periodic.
// ub_trace[s] receives the bulk velocity measured by channel_cfr at each
// sub-step (before its correction).
int ox_run_channel(void* h, double* ux_, double* uy_, double* uz_, int nsteps, double dt, double xnu, int itimescheme,
                   double wrotation, int spinup_time, double* ub_trace, double* divmax) {
  const OxCtx* c = (const OxCtx*)h;
  if (!(c->ax[0].periodic && !c->ax[1].periodic && c->ax[2].periodic)) return -2;
  if (c->ax[1].ncl1 != 2 || c->ax[1].ncln != 2) return -2;
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const size_t N = (size_t)nx * ny * nz;
  vec ux(ux_, ux_ + N), uy(uy_, uy_ + N), uz(uz_, uz_ + N);
  const int ntime = (itimescheme == 3) ? 3 : 2;
  std::vector<vec> dux(ntime, vec(N, 0.0)), duy(ntime, vec(N, 0.0)), duz(ntime, vec(N, 0.0));
  double adt[3] = {0, 0, 0}, bdt[3] = {0, 0, 0}, cdt[3] = {0, 0, 0}, gdt[3] = {0, 0, 0};
  int nsub = 1;
  if (itimescheme == 3) {
    adt[0] = (23.0 / 12.0) * dt; bdt[0] = -(16.0 / 12.0) * dt; cdt[0] = (5.0 / 12.0) * dt;
    gdt[0] = adt[0] + bdt[0] + cdt[0];
  } else if (itimescheme == 5) {
    nsub = 3;
    adt[0] = (8.0 / 15.0) * dt; bdt[0] = 0; gdt[0] = adt[0];
    adt[1] = (5.0 / 12.0) * dt; bdt[1] = (-17.0 / 60.0) * dt; gdt[1] = adt[1] + bdt[1];
    adt[2] = (3.0 / 4.0) * dt; bdt[2] = (-5.0 / 12.0) * dt; gdt[2] = adt[2] + bdt[2];
  } else {
    return -3;
  }
  // wall pressure gradients dpdxy1, dpdzy1 (j = 1) and dpdxyn, dpdzyn (j = ny)
  vec dpdxy1((size_t)nx * nz, 0.0), dpdzy1(dpdxy1.size(), 0.0), dpdxyn(dpdxy1.size(), 0.0),
      dpdzyn(dpdxy1.size(), 0.0);
  vec pp3, px(N), py(N), pz(N);
  const double dy = c->ax[1].d;
  const double coeff = dy / (c->yly * (double)(nx * nz));
  int s = 0;
  for (int itime = 1; itime <= nsteps; ++itime) {
    for (int itr = 1; itr <= nsub; ++itr) {
      // channel_cfr
      double ub = 0.0;
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) ub = ub + ux[idx3(i, j, k, nx, ny)] / c->ppy[j];
      ub = ub * coeff;
      const double can = -(2.0 / 3.0 - ub);
      for (size_t m = 0; m < N; ++m) ux[m] = ux[m] - can;
      if (ub_trace) ub_trace[s] = ub;
      ++s;
      momentum_rhs(*c, ux, uy, uz, xnu, dux[0], duy[0], duz[0]);
      if (itime < spinup_time) {
        for (size_t m = 0; m < N; ++m) {
          dux[0][m] = dux[0][m] - wrotation * uy[m];
          duy[0][m] = duy[0][m] + wrotation * ux[m];
        }
      }
      vec* vars[3] = {&ux, &uy, &uz};
      std::vector<vec>* dvs[3] = {&dux, &duy, &duz};
      for (int q = 0; q < 3; ++q) {
        vec& v = *vars[q];
        std::vector<vec>& d = *dvs[q];
        if (itimescheme == 3) {
          if (itime == 1) {
            for (size_t m = 0; m < N; ++m) v[m] = dt * d[0][m] + v[m];
          } else if (itime == 2) {
            for (size_t m = 0; m < N; ++m) v[m] = 1.5 * dt * d[0][m] - 0.5 * dt * d[1][m] + v[m];
            d[2] = d[1];
          } else {
            for (size_t m = 0; m < N; ++m)
              v[m] = adt[0] * d[0][m] + bdt[0] * d[1][m] + cdt[0] * d[2][m] + v[m];
            d[2] = d[1];
          }
          d[1] = d[0];
        } else {
          if (itr == 1) {
            for (size_t m = 0; m < N; ++m) v[m] = gdt[0] * d[0][m] + v[m];
          } else {
            for (size_t m = 0; m < N; ++m) v[m] = adt[itr - 1] * d[0][m] + bdt[itr - 1] * d[1][m] + v[m];
          }
          d[1] = d[0];
        }
      }
      // pre_correc: no-slip walls with the stored tangential pressure gradient
      const double g = gdt[itr - 1];
      for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
          const size_t w = (size_t)i + (size_t)nx * k;
          dpdxy1[w] = dpdxy1[w] * g;
          dpdzy1[w] = dpdzy1[w] * g;
          dpdxyn[w] = dpdxyn[w] * g;
          dpdzyn[w] = dpdzyn[w] * g;
          ux[idx3(i, 0, k, nx, ny)] = 0.0 + dpdxy1[w];
          uy[idx3(i, 0, k, nx, ny)] = 0.0;
          uz[idx3(i, 0, k, nx, ny)] = 0.0 + dpdzy1[w];
          ux[idx3(i, ny - 1, k, nx, ny)] = 0.0 + dpdxyn[w];
          uy[idx3(i, ny - 1, k, nx, ny)] = 0.0;
          uz[idx3(i, ny - 1, k, nx, ny)] = 0.0 + dpdzyn[w];
        }
      divergence(*c, ux, uy, uz, pp3);
      poisson_010(*c, pp3.data());
      gradp(*c, pp3, px, py, pz);
      for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
          const size_t w = (size_t)i + (size_t)nx * k;
          dpdxy1[w] = px[idx3(i, 0, k, nx, ny)] / g;
          dpdzy1[w] = pz[idx3(i, 0, k, nx, ny)] / g;
          dpdxyn[w] = px[idx3(i, ny - 1, k, nx, ny)] / g;
          dpdzyn[w] = pz[idx3(i, ny - 1, k, nx, ny)] / g;
        }
      for (size_t m = 0; m < N; ++m) { ux[m] = ux[m] - px[m]; uy[m] = uy[m] - py[m]; uz[m] = uz[m] - pz[m]; }
    }
  }
  if (divmax) {
    vec p;
    divergence(*c, ux, uy, uz, p);
    double dmax = 0;
    for (double v : p) dmax = std::max(dmax, std::fabs(v));
    *divmax = dmax;
  }
  std::memcpy(ux_, ux.data(), N * sizeof(double));
  std::memcpy(uy_, uy.data(), N * sizeof(double));
  std::memcpy(uz_, uz.data(), N * sizeof(double));
  return s;
}

}  // extern "C"
