"""ctypes front end of the C++ oracle (test infrastructure only).

Arrays are numpy float64 in C order with shape (nz, ny, nx), which is the
reference's Fortran (nx, ny, nz) layout with x fastest.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

OP_DER1, OP_DER2, OP_FIL, OP_DVP, OP_IVP, OP_DPV, OP_IPV = range(7)

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "x3d_oracle.cpp")
_OUT = os.path.join(_HERE, "_build", "libx3d_oracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile the oracle with g++ (OpenMP, no FMA contraction)."""
    os.makedirs(os.path.dirname(_OUT), exist_ok=True)
    if (not force and os.path.exists(_OUT)
            and os.path.getmtime(_OUT) >= os.path.getmtime(_SRC)):
        return _OUT
    tmp = _OUT + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
           "-shared", "-o", tmp, _SRC]
    subprocess.check_call(cmd)
    os.replace(tmp, _OUT)
    return _OUT


def _load():
    global _lib
    with _lock:
        if _lib is None:
            lib = ctypes.CDLL(build())
            P = ctypes.c_void_p
            D = ctypes.POINTER(ctypes.c_double)
            I = ctypes.POINTER(ctypes.c_int)
            lib.ox_create.restype = P
            lib.ox_create.argtypes = [I, D]
            lib.ox_destroy.argtypes = [P]
            lib.ox_set_threads.argtypes = [ctypes.c_int]
            lib.ox_op.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, D, D, I, D]
            lib.ox_coeffs.argtypes = [P, ctypes.c_int, ctypes.c_int, D]
            lib.ox_scalars.argtypes = [P, ctypes.c_int, D]
            lib.ox_poisson.argtypes = [P, D]
            lib.ox_divergence.argtypes = [P, D, D, D, D]
            lib.ox_gradp.argtypes = [P, D, D, D, D]
            lib.ox_rhs.argtypes = [P, D, D, D, ctypes.c_double, D, D, D]
            lib.ox_tgv_stats.argtypes = [P, D, D, D, ctypes.c_double, D]
            lib.ox_run.argtypes = [P, D, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_int, ctypes.c_int, D, D]
            lib.ox_stretching.argtypes = [P, ctypes.c_int, D]
            lib.ox_set_les.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double]
            lib.ox_les.argtypes = [P, D, D, D, D, D, D, D]
            lib.ox_run_channel.argtypes = [P, D, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int, ctypes.c_double, ctypes.c_int, D, D]
            _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """Grid + numerics options, mirroring the reference's namelist subset."""

    def __init__(self, nx, ny, nz, xlx, yly, zlz, bc=((0, 0), (0, 0), (0, 0)),
                 ifirstder=4, isecondder=4, ipinter=3, filter_alpha=0.49,
                 nu0nu=4.0, cnu=0.44, istret=0, beta=0.0):
        self.lib = _load()
        self.nx, self.ny, self.nz = nx, ny, nz
        self.bc = bc
        self.istret = istret
        iv = (ctypes.c_int * 13)(nx, ny, nz, bc[0][0], bc[0][1], bc[1][0], bc[1][1],
                                  bc[2][0], bc[2][1], ifirstder, isecondder, ipinter, istret)
        dv = (ctypes.c_double * 7)(xlx, yly, zlz, filter_alpha, nu0nu, cnu, beta)
        self.h = self.lib.ox_create(iv, dv)
        self.n = (nx, ny, nz)
        self.nm = tuple(n if b == (0, 0) else n - 1 for n, b in zip(self.n, bc))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.ox_destroy(h)
            self.h = None

    @staticmethod
    def set_threads(n):
        return _load().ox_set_threads(int(n))

    def op(self, axis, op, npaire, u, pp=None):
        """Apply operator `op` along `axis` (0=x,1=y,2=z) to u (shape (nz,ny,nx))."""
        u = _c64(u)
        dims = [u.shape[2], u.shape[1], u.shape[0]]
        nout = dims[axis]
        if op in (OP_DVP, OP_IVP):
            nout = self.nm[axis]
        elif op in (OP_DPV, OP_IPV):
            nout = self.n[axis]
        od = list(dims)
        od[axis] = nout
        t = np.empty((od[2], od[1], od[0]), dtype=np.float64)
        di = (ctypes.c_int * 3)(*dims)
        ppp = _dp(_c64(pp)) if pp is not None else None
        rc = self.lib.ox_op(self.h, axis, op, npaire, _dp(u), _dp(t), di, ppp)
        assert rc == 0
        return t

    def coeffs(self, axis, which):
        out = np.zeros(max(self.n) + 8, dtype=np.float64)
        n = self.lib.ox_coeffs(self.h, axis, which, _dp(out))
        assert n >= 0
        return out[:n].copy()

    def scalars(self, axis):
        out = np.zeros(64, dtype=np.float64)
        n = self.lib.ox_scalars(self.h, axis, _dp(out))
        names = ["alfai", "afi", "bfi", "alsai", "asi", "bsi", "csi", "dsi", "fiali", "fiai",
                 "fibi", "fici", "fidi", "alcai6", "aci6", "bci6", "ailcai6", "aici6", "bici6",
                 "cici6", "dici6", "d"]
        return dict(zip(names, out[:n]))

    def poisson(self, rhs):
        r = _c64(rhs).copy()
        rc = self.lib.ox_poisson(self.h, _dp(r))
        assert rc == 0, rc
        return r

    def divergence(self, ux, uy, uz):
        nxm, nym, nzm = self.nm
        out = np.empty((nzm, nym, nxm))
        self.lib.ox_divergence(self.h, _dp(_c64(ux)), _dp(_c64(uy)), _dp(_c64(uz)), _dp(out))
        return out

    def gradp(self, pp3):
        shp = (self.nz, self.ny, self.nx)
        px, py, pz = np.empty(shp), np.empty(shp), np.empty(shp)
        self.lib.ox_gradp(self.h, _dp(_c64(pp3)), _dp(px), _dp(py), _dp(pz))
        return px, py, pz

    def rhs(self, ux, uy, uz, xnu):
        shp = (self.nz, self.ny, self.nx)
        hx, hy, hz = np.empty(shp), np.empty(shp), np.empty(shp)
        self.lib.ox_rhs(self.h, _dp(_c64(ux)), _dp(_c64(uy)), _dp(_c64(uz)), xnu,
                        _dp(hx), _dp(hy), _dp(hz))
        return hx, hy, hz

    def tgv_stats(self, ux, uy, uz, xnu):
        out = np.zeros(4)
        self.lib.ox_tgv_stats(self.h, _dp(_c64(ux)), _dp(_c64(uy)), _dp(_c64(uz)), xnu, _dp(out))
        return out

    def run(self, ux, uy, uz, nsteps, dt, xnu, itimescheme=3, every=10):
        ux, uy, uz = _c64(ux).copy(), _c64(uy).copy(), _c64(uz).copy()
        rows = max(1, nsteps // max(every, 1))
        stats = np.zeros((rows, 5))
        dmax = np.zeros(1)
        n = self.lib.ox_run(self.h, _dp(ux), _dp(uy), _dp(uz), nsteps, dt, xnu, itimescheme,
                            every, _dp(stats), _dp(dmax))
        assert n >= 0, n
        return ux, uy, uz, stats[:n], float(dmax[0])

    STRETCH_NAMES = ("yp", "ypi", "ppy", "pp2y", "pp4y", "ppyi", "pp2yi", "pp4yi")

    def stretching(self):
        """Mesh metrics of src/stretching.f90 (dict of arrays) plus alpha."""
        out = {}
        buf = np.zeros(self.ny + 8)
        for w, nm in enumerate(self.STRETCH_NAMES):
            n = self.lib.ox_stretching(self.h, w, _dp(buf))
            out[nm] = buf[:n].copy()
        self.lib.ox_stretching(self.h, 8, _dp(buf))
        out["alpha"] = float(buf[0])
        return out

    def run_channel(self, ux, uy, uz, nsteps, dt, xnu, itimescheme=5, wrotation=0.0, spinup_time=0):
        """Channel time loop (constant flow rate, no-slip walls in y); returns the
        velocity, the bulk velocity seen by the flow-rate correction at every
        sub-step, and max|div u| at the end."""
        ux, uy, uz = _c64(ux).copy(), _c64(uy).copy(), _c64(uz).copy()
        nsub = 3 if itimescheme == 5 else 1
        ub = np.zeros(nsteps * nsub)
        dmax = np.zeros(1)
        n = self.lib.ox_run_channel(self.h, _dp(ux), _dp(uy), _dp(uz), nsteps, dt, xnu, itimescheme,
                                    wrotation, spinup_time, _dp(ub), _dp(dmax))
        assert n >= 0, n
        return ux, uy, uz, ub[:n], float(dmax[0])

    def set_les(self, jles, smagcst=0.14, maxdsmagcst=0.3):
        """Explicit LES model in the right-hand side: 1 Smagorinsky, 3 dynamic."""
        assert self.lib.ox_set_les(self.h, jles, smagcst, maxdsmagcst) == 0

    def les(self, ux, uy, uz):
        """(nut, sgsx, sgsy, sgsz) of compute_SGS for the current model."""
        shp = (self.nz, self.ny, self.nx)
        out = [np.empty(shp) for _ in range(4)]
        rc = self.lib.ox_les(self.h, _dp(_c64(ux)), _dp(_c64(uy)), _dp(_c64(uz)), *[_dp(o) for o in out])
        assert rc == 0, rc
        return out
