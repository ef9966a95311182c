"""Host-side mirror of the reference's operator interfaces, over the C ABI.

`Context` corresponds to the reference's init-time state (schemes(),
filter(), decomp_2d_poisson_init).  Its methods carry the reference's routine
names and argument meaning (src/module_param.f90:135-233 for the derivative
and filter interfaces, src/derive.f90:3796-5615 for the staggered operators,
src/poisson.f90:57-62 for poisson).  Fields are torch CUDA tensors of shape
(nz, ny, nx), i.e. the reference's Fortran (nx, ny, nz) layout with x fastest;
every call runs the CUDA kernels of libx3dgpu.so on the current torch stream.
Coefficient vectors, where the reference passes them, may be given as numpy
arrays (they must be one of the context's sets) or omitted.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (COEF, OP_DER1, OP_DER2, OP_DPV, OP_DVP, OP_FIL, OP_IPV, OP_IVP,  # noqa: F401
                   PREC_FP64, PREC_MIXED, check)


def _torch():
    import torch
    return torch


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _hptr(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.ctypes.data_as(ctypes.c_void_p), a


def _dev(t, dtype=None):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("fields must be CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("fields must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError("expected %s, got %s" % (dtype, t.dtype))
    return t


class Context:
    """Grid + numerical options; owns the coefficient tables in HBM."""

    def __init__(self, nx, ny, nz, xlx, yly, zlz, bc=((0, 0), (0, 0), (0, 0)), ifirstder=4,
                 isecondder=4, ipinter=3, filter_alpha=0.49, nu0nu=4.0, cnu=0.44, istret=0, beta=0.0):
        self.lib = _lib.load()
        g = _lib.Grid(nx, ny, nz, xlx, yly, zlz, bc[0][0], bc[0][1], bc[1][0], bc[1][1],
                      bc[2][0], bc[2][1], istret, beta)
        o = _lib.NumOpts(ifirstder, isecondder, ipinter, filter_alpha, nu0nu, cnu)
        h = ctypes.c_void_p()
        check(self.lib.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)), "x3d_ctx_create")
        self.h = h
        self.n = (nx, ny, nz)
        self.L = (xlx, yly, zlz)
        self.istret, self.beta = istret, beta
        self.bc = bc
        self.nm = tuple(n if b == (0, 0) else n - 1 for n, b in zip(self.n, bc))

    def close(self):
        if getattr(self, "h", None):
            self.lib.x3d_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    STRETCH_NAMES = ("yp", "ypi", "ppy", "pp2y", "pp4y", "ppyi", "pp2yi", "pp4yi")

    def stretching(self):
        """y-mesh metrics (dict of host arrays) and the mapping constant alpha."""
        out = {}
        buf = np.zeros(self.n[1] + 8)
        for w, nm in enumerate(self.STRETCH_NAMES):
            k = check(self.lib.x3d_get_stretching(self.h, w, buf.ctypes.data_as(ctypes.c_void_p), buf.size),
                      "x3d_get_stretching")
            out[nm] = buf[:k].copy()
        check(self.lib.x3d_get_stretching(self.h, 8, buf.ctypes.data_as(ctypes.c_void_p), buf.size),
              "x3d_get_stretching")
        out["alpha"] = float(buf[0])
        return out

    # ---- coefficient vectors (host copies, as the reference passes them) ----
    def coeffs(self, axis, name):
        out = np.zeros(max(self.n) + 8)
        n = check(self.lib.x3d_get_coeffs(self.h, axis, COEF[name.upper()],
                                          out.ctypes.data_as(ctypes.c_void_p), out.size), "x3d_get_coeffs")
        return out[:n].copy()

    # ---- generic entry -------------------------------------------------------
    def out_shape(self, axis, op, shape):
        nz, ny, nx = shape
        d = [nx, ny, nz]
        if op in (OP_DVP, OP_IVP):
            d[axis] = self.nm[axis]
        elif op in (OP_DPV, OP_IPV):
            d[axis] = self.n[axis]
        return (d[2], d[1], d[0])

    def apply(self, axis, op, npaire, u, out=None, coefset=-1):
        torch = _torch()
        u = _dev(u)
        dtype = {torch.float64: 0, torch.float32: 1}.get(u.dtype)
        if dtype is None:
            raise TypeError("float64 or float32 fields only")
        if out is None:
            out = torch.empty(self.out_shape(axis, op, u.shape), dtype=u.dtype, device=u.device)
        dims = (ctypes.c_int * 3)(u.shape[2], u.shape[1], u.shape[0])
        check(self.lib.x3d_apply(self.h, axis, op, npaire, coefset, dtype, _ptr(out), _ptr(u), dims, _stream()),
              "x3d_apply")
        return out

    def conv_diff(self, axis, q, uj, uq, a1=None, nu=1.0, out=None):
        """One direction's share of the momentum right-hand side of u_q
        (binary32, fused kernel): nu d_jj u_q + a1 - (d_j(u_j u_q) + u_j d_j u_q) / 2."""
        torch = _torch()
        uj = _dev(uj, torch.float32)
        uq = _dev(uq, torch.float32)
        if a1 is not None:
            _dev(a1, torch.float32)
        if out is None:
            out = torch.empty_like(uq)
        dims = (ctypes.c_int * 3)(uq.shape[2], uq.shape[1], uq.shape[0])
        check(self.lib.x3d_conv_diff_f32(self.h, axis, q, _ptr(out), _ptr(uj), _ptr(uq),
                                         None if a1 is None else _ptr(a1), ctypes.c_float(nu), dims, _stream()),
              "x3d_conv_diff_f32")
        return out

    # ---- reference-named routines (FP64) -------------------------------------
    def _colloc(self, fn, t, u, f, s, w, nx, ny, nz, npaire, *pp):
        torch = _torch()
        _dev(t, torch.float64)
        _dev(u, torch.float64)
        hs = [_hptr(a) for a in (f, s, w)]
        args = [h[0] if h else None for h in hs]
        check(fn(self.h, _ptr(t), _ptr(u), None, None, *args, *pp, nx, ny, nz, npaire, 0.0, _stream()),
              fn.__name__)
        return t

    def derx(self, tx, ux, rx=None, sx=None, ffx=None, fsx=None, fwx=None, nx=None, ny=None, nz=None,
             npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_derx, tx, ux, ffx, fsx, fwx, nx, ny, nz, npaire)

    def dery(self, ty, uy, ry=None, sy=None, ffy=None, fsy=None, fwy=None, ppy=None, nx=None, ny=None,
             nz=None, npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        hp = _hptr(ppy)  # NULL: the context's ppy (applied only on a stretched mesh)
        return self._colloc(self.lib.x3d_dery, ty, uy, ffy, fsy, fwy, nx, ny, nz, npaire, hp[0] if hp else None)

    def derz(self, tz, uz, rz=None, sz=None, ffz=None, fsz=None, fwz=None, nx=None, ny=None, nz=None,
             npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_derz, tz, uz, ffz, fsz, fwz, nx, ny, nz, npaire)

    def derxx(self, tx, ux, rx=None, sx=None, sfx=None, ssx=None, swx=None, nx=None, ny=None, nz=None,
              npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_derxx, tx, ux, sfx, ssx, swx, nx, ny, nz, npaire)

    def deryy(self, ty, uy, ry=None, sy=None, sfy=None, ssy=None, swy=None, nx=None, ny=None, nz=None,
              npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_deryy, ty, uy, sfy, ssy, swy, nx, ny, nz, npaire)

    def derzz(self, tz, uz, rz=None, sz=None, sfz=None, ssz=None, swz=None, nx=None, ny=None, nz=None,
              npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_derzz, tz, uz, sfz, ssz, swz, nx, ny, nz, npaire)

    def filx(self, tx, ux, rx=None, fisx=None, fiffx=None, fifsx=None, fifwx=None, nx=None, ny=None,
             nz=None, npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_filx, tx, ux, fiffx, fifsx, fifwx, nx, ny, nz, npaire)

    def fily(self, ty, uy, ry=None, fisy=None, fiffy=None, fifsy=None, fifwy=None, nx=None, ny=None,
             nz=None, npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_fily, ty, uy, fiffy, fifsy, fifwy, nx, ny, nz, npaire)

    def filz(self, tz, uz, rz=None, fisz=None, fiffz=None, fifsz=None, fifwz=None, nx=None, ny=None,
             nz=None, npaire=0, lind=0.0):
        nx, ny, nz = self._dims(nx, ny, nz)
        return self._colloc(self.lib.x3d_filz, tz, uz, fiffz, fifsz, fifwz, nx, ny, nz, npaire)

    def _dims(self, nx, ny, nz):
        return (nx or self.n[0], ny or self.n[1], nz or self.n[2])

    # ---- Poisson / projection ------------------------------------------------
    def poisson(self, rhs, precision=0):
        torch = _torch()
        _dev(rhs, torch.float64)
        check(self.lib.x3d_poisson_ex(self.h, _ptr(rhs), precision, _stream()), "x3d_poisson")
        return rhs

    def poisson_noalloc(self, rhs):
        """x3d_poisson_noalloc: same solve as poisson(), with all scratch in the
        library's fixed device array (no allocation; grids up to its size)."""
        torch = _torch()
        _dev(rhs, torch.float64)
        check(self.lib.x3d_poisson_noalloc(self.h, _ptr(rhs), _stream()), "x3d_poisson_noalloc")
        return rhs

    def divergence(self, ux, uy, uz, pp3=None):
        """divergence of (ux, uy, uz) on the pressure mesh, FP64 result; binary32
        velocity runs the FP32 operators (x3d_divergence_f32)."""
        torch = _torch()
        if pp3 is None:
            pp3 = torch.empty((self.nm[2], self.nm[1], self.nm[0]), dtype=torch.float64, device=ux.device)
        fn = self.lib.x3d_divergence_f32 if ux.dtype == torch.float32 else self.lib.x3d_divergence
        for t in (ux, uy, uz):
            _dev(t, ux.dtype)
        _dev(pp3, torch.float64)
        check(fn(self.h, _ptr(pp3), _ptr(ux), _ptr(uy), _ptr(uz), _stream()), fn.__name__)
        return pp3

    def gradp(self, pp3, px=None, py=None, pz=None):
        """gradient of pp3 on the velocity mesh in pp3's precision (FP32 runs
        x3d_gradp_f32)."""
        torch = _torch()
        shp = (self.n[2], self.n[1], self.n[0])
        dt = pp3.dtype
        px = torch.empty(shp, dtype=dt, device=pp3.device) if px is None else px
        py = torch.empty(shp, dtype=dt, device=pp3.device) if py is None else py
        pz = torch.empty(shp, dtype=dt, device=pp3.device) if pz is None else pz
        for t in (px, py, pz):
            _dev(t, dt)
        fn = self.lib.x3d_gradp_f32 if dt == torch.float32 else self.lib.x3d_gradp
        check(fn(self.h, _ptr(px), _ptr(py), _ptr(pz), _ptr(pp3), _stream()), fn.__name__)
        return px, py, pz

    def cor_vel(self, ux, uy, uz, px, py, pz):
        check(self.lib.x3d_cor_vel(self.h, _ptr(ux), _ptr(uy), _ptr(uz), _ptr(px), _ptr(py), _ptr(pz),
                                   _stream()), "x3d_cor_vel")
        return ux, uy, uz


class Solver:
    """Resident incompressible solver (time loop body of src/xcompact3d.f90:29-102)."""

    def __init__(self, ctx, dt, xnu, itimescheme=3, precision=PREC_FP64):
        self.ctx = ctx
        self.lib = ctx.lib
        self.itimescheme, self.dt, self.xnu = itimescheme, dt, xnu
        o = _lib.SolverOpts(itimescheme, dt, xnu, precision)
        h = ctypes.c_void_p()
        check(self.lib.x3d_solver_create(ctx.h, ctypes.byref(o), ctypes.byref(h)), "x3d_solver_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.x3d_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_velocity(self, ux, uy, uz):
        """ux, uy, uz: numpy float64 (host), contiguous torch CPU float64 (host;
        page-locked ones are read by the kernels directly) or torch CUDA float64
        (device)."""
        if isinstance(ux, np.ndarray):
            a = [np.ascontiguousarray(v, dtype=np.float64) for v in (ux, uy, uz)]
            check(self.lib.x3d_solver_set_velocity(self.h, *[v.ctypes.data_as(ctypes.c_void_p) for v in a], 0),
                  "x3d_solver_set_velocity")
        else:
            on_dev = 1 if ux.is_cuda else 0
            check(self.lib.x3d_solver_set_velocity(self.h, _ptr(ux), _ptr(uy), _ptr(uz), on_dev),
                  "x3d_solver_set_velocity")

    def get_velocity(self):
        nx, ny, nz = self.ctx.n
        out = [np.empty((nz, ny, nx)) for _ in range(3)]
        check(self.lib.x3d_solver_get_velocity(self.h, *[v.ctypes.data_as(ctypes.c_void_p) for v in out], 0),
              "x3d_solver_get_velocity")
        return out

    def get_velocity_into(self, ux, uy, uz):
        """Copy the velocity into caller-provided host (numpy or pinned torch CPU)
        or CUDA float64 arrays."""
        def addr(a):
            return a.ctypes.data_as(ctypes.c_void_p) if isinstance(a, np.ndarray) else ctypes.c_void_p(a.data_ptr())
        on_dev = 0 if isinstance(ux, np.ndarray) or not getattr(ux, "is_cuda", False) else 1
        check(self.lib.x3d_solver_get_velocity(self.h, addr(ux), addr(uy), addr(uz), on_dev),
              "x3d_solver_get_velocity")

    def set_channel(self, target_ub=2.0 / 3.0, wrotation=0.0, spinup_time=0):
        """Channel case: constant flow rate control and the spin-up rotation."""
        check(self.lib.x3d_solver_set_channel(self.h, target_ub, wrotation, spinup_time),
              "x3d_solver_set_channel")

    def get_field(self, which):
        """Restart state slot as a host array: 0..2 velocity, 3..5 / 6..8 the
        AB history, 9 the pressure (pressure mesh)."""
        nx, ny, nz = self.ctx.n
        shp = (nz, ny, nx) if which != 9 else tuple(reversed(self.ctx.nm))
        out = np.empty(shp)
        check(self.lib.x3d_solver_get_field(self.h, which, out.ctypes.data_as(ctypes.c_void_p), 0),
              "x3d_solver_get_field")
        return out

    def set_field(self, which, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        check(self.lib.x3d_solver_set_field(self.h, which, a.ctypes.data_as(ctypes.c_void_p), 0),
              "x3d_solver_set_field")

    def set_itime(self, itime):
        check(self.lib.x3d_solver_set_itime(self.h, int(itime)), "x3d_solver_set_itime")

    @property
    def itime(self):
        return check(self.lib.x3d_solver_get_itime(self.h), "x3d_solver_get_itime")

    def set_les(self, jles, smagcst=0.14, maxdsmagcst=0.3):
        """Explicit LES model: 1 Smagorinsky, 3 dynamic Smagorinsky, 0 off."""
        check(self.lib.x3d_solver_set_les(self.h, jles, smagcst, maxdsmagcst), "x3d_solver_set_les")

    def les_fields(self):
        """(nut, sgsx, sgsy, sgsz) of the current velocity, as CUDA tensors."""
        torch = _torch()
        nx, ny, nz = self.ctx.n
        out = [torch.empty((nz, ny, nx), dtype=torch.float64, device="cuda") for _ in range(4)]
        check(self.lib.x3d_solver_les_fields(self.h, *[_ptr(o) for o in out], _stream()), "x3d_solver_les_fields")
        return out

    def bulk_velocity(self):
        """Bulk velocity seen by the flow-rate control at each sub-step of the last step."""
        out = np.zeros(8)
        n = check(self.lib.x3d_solver_bulk_velocity(self.h, out.ctypes.data_as(ctypes.c_void_p), out.size),
                  "x3d_solver_bulk_velocity")
        return out[:n].copy()

    def init_tgv(self):
        check(self.lib.x3d_solver_init_tgv(self.h), "x3d_solver_init_tgv")

    def step(self, nsteps=1, stream=None):
        st = _stream() if stream is None else stream
        check(self.lib.x3d_solver_step(self.h, nsteps, st), "x3d_solver_step")

    def tgv_stats(self):
        out = np.zeros(4)
        check(self.lib.x3d_solver_tgv_stats(self.h, out.ctypes.data_as(ctypes.c_void_p), _stream()),
              "x3d_solver_tgv_stats")
        return out

    def divmax(self):
        out = np.zeros(1)
        check(self.lib.x3d_solver_divmax(self.h, out.ctypes.data_as(ctypes.c_void_p), _stream()),
              "x3d_solver_divmax")
        return float(out[0])

    def launches_per_step(self):
        return self.lib.x3d_solver_launches_per_step(self.h)
