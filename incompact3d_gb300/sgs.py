"""Learned subgrid-stress closure for the TGV LES (FP32 MLP on the GPU).

The model maps the 9 resolved velocity gradients du_i/dx_j and the filter
width to the 6 subgrid stresses tau_ij; it is trained on box-filtered (ratio
4) snapshots of a DNS run by this package's own solver and then used inside
the LES time step (``Solver.set_les_mlp``).  The dynamic Smagorinsky model of
the reference (src/les_models.f90:333-903) is the fallback and the cost
baseline, and the box-filtered DNS is the judge of the model's error.

All compute runs in libx3dgpu's kernels (solver, box filter, MLP training and
inference); PyTorch only holds device buffers and shuffles sample indices.
"""
import ctypes
import math
import time

import numpy as np

from . import _lib
from ._lib import check
from .operators import OP_DER1, Context, Solver, _torch

NIN, NHID, NOUT = 10, 64, 6


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


class Mlp:
    """The 10-64-64-6 GELU network (parameters and Adam state on the device)."""

    def __init__(self, seed=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.x3d_mlp_create(NIN, NHID, NOUT, ctypes.byref(h)), "x3d_mlp_create")
        self.h = h
        self.nparam = self.lib.x3d_mlp_param_count()
        self.set(init_params(seed), np.ones(NIN + NOUT, dtype=np.float32))

    def close(self):
        if getattr(self, "h", None):
            self.lib.x3d_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, params=None, scales=None):
        pp = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        ss = None if scales is None else np.ascontiguousarray(scales, dtype=np.float32)
        check(self.lib.x3d_mlp_set_params(self.h, None if pp is None else pp.ctypes.data_as(ctypes.c_void_p),
                                          None if ss is None else ss.ctypes.data_as(ctypes.c_void_p)),
              "x3d_mlp_set_params")

    def get(self):
        p = np.empty(self.nparam, dtype=np.float32)
        s = np.empty(NIN + NOUT, dtype=np.float32)
        check(self.lib.x3d_mlp_get_params(self.h, p.ctypes.data_as(ctypes.c_void_p),
                                          s.ctypes.data_as(ctypes.c_void_p)), "x3d_mlp_get_params")
        return p, s

    def infer(self, X):
        torch = _torch()
        Y = torch.empty((X.shape[0], NOUT), dtype=torch.float32, device=X.device)
        check(self.lib.x3d_mlp_infer(self.h, _p(X), _p(Y), X.shape[0], None), "x3d_mlp_infer")
        return Y

    def train_step(self, X, T, lr, want_loss=False):
        loss = ctypes.c_float(0.0)
        check(self.lib.x3d_mlp_train_step(self.h, _p(X), _p(T), X.shape[0], ctypes.c_float(lr),
                                          ctypes.byref(loss) if want_loss else None, None),
              "x3d_mlp_train_step")
        return loss.value if want_loss else None


def init_params(seed=0):
    """Glorot-uniform weights, zero biases, in the library's layout."""
    rng = np.random.default_rng(seed)

    def glorot(o, i):
        a = math.sqrt(6.0 / (i + o))
        return rng.uniform(-a, a, size=(o, i)).astype(np.float32)

    parts = [glorot(NHID, NIN).ravel(), np.zeros(NHID, np.float32), glorot(NHID, NHID).ravel(),
             np.zeros(NHID, np.float32), glorot(NOUT, NHID).ravel(), np.zeros(NOUT, np.float32)]
    return np.concatenate(parts)


def box_filter4(lib, ux, uy, uz):
    """Filtered velocity (3 fields) and tau_ij (6 fields) on the /4 grid."""
    torch = _torch()
    nz, ny, nx = ux.shape
    shp = (nz // 4, ny // 4, nx // 4)
    ub = [torch.empty(shp, dtype=torch.float64, device=ux.device) for _ in range(3)]
    tau = torch.empty((6,) + shp, dtype=torch.float64, device=ux.device)
    check(lib.x3d_box_filter4(_p(ux), _p(uy), _p(uz), nx, ny, nz, _p(ub[0]), _p(ub[1]), _p(ub[2]), _p(tau), None),
          "x3d_box_filter4")
    return ub, tau


def gradients(ctx, u):
    """du_i/dx_j (i-major) of a velocity on ctx's grid, compact first
    derivatives with the parities the reference uses for them."""
    g = []
    for i in range(3):
        for j in range(3):
            g.append(ctx.apply(j, OP_DER1, 0 if i == j else 1, u[i]))
    return g


def features(ctx, u):
    torch = _torch()
    g = gradients(ctx, u)
    n = g[0].numel()
    delta = (ctx.L[0] / ctx.n[0] * ctx.L[1] / ctx.n[1] * ctx.L[2] / ctx.n[2]) ** (1.0 / 3.0)
    X = torch.empty((n, NIN), dtype=torch.float32, device=u[0].device)
    for q in range(9):
        X[:, q] = g[q].reshape(-1).float()
    X[:, 9] = delta
    return X, delta


def _stats(torch, s):
    e = 0.5 * sum(float((u * u).mean()) for u in s)
    return e


def run_pipeline(n_dns=512, n_les=128, re=5000.0, dt=0.002, t_end=20.0, t_train=(2.0, 10.0), snap_every=1.0,
                 epochs=3, batch=16384, lr=1e-3, record_every=10, seed=0, log=print):
    """DNS -> box-filtered training set -> MLP training -> LES comparison.

    Returns a dict: filtered-DNS and LES kinetic energy / dissipation histories,
    the dissipation errors of the learned and the dynamic-Smagorinsky LES
    against the filtered DNS, step costs, and the training / validation loss."""
    torch = _torch()
    L = 2 * math.pi
    xnu = 1.0 / re
    lib = _lib.load()
    out = {"n_dns": n_dns, "n_les": n_les, "re": re, "dt": dt, "t_end": t_end}
    # ---- DNS with box-filtered statistics and training snapshots ----------
    cd = Context(n_dns, n_dns, n_dns, L, L, L)
    cl = Context(n_les, n_les, n_les, L, L, L)
    sd = Solver(cd, dt, xnu, itimescheme=3, precision=_lib.PREC_MIXED)
    sd.init_tgv()
    shp = (n_dns, n_dns, n_dns)
    u = [torch.empty(shp, dtype=torch.float64, device="cuda") for _ in range(3)]
    nsteps = int(round(t_end / dt))
    snaps = set(int(round(t / dt)) for t in np.arange(t_train[0], t_train[1] + 1e-9, snap_every))
    Xs, Ts, tdns, edns = [], [], [], []
    t0 = time.time()
    for it in range(0, nsteps + 1):
        if it % record_every == 0 or it in snaps:
            sd.get_velocity_into(*u)
            ub, tau = box_filter4(lib, *u)
            if it % record_every == 0:
                tdns.append(it * dt)
                edns.append(_stats(torch, ub))
            if it in snaps:
                X, delta = features(cl, ub)
                Xs.append(X)
                Ts.append(tau.reshape(6, -1).t().contiguous().float())
        if it < nsteps:
            sd.step(1)
    torch.cuda.synchronize()
    out["dns_seconds"] = time.time() - t0
    sd.close()
    del u
    # ---- training ------------------------------------------------------------
    Xtr = torch.cat(Xs[:-1]) if len(Xs) > 1 else Xs[0]
    Ttr = torch.cat(Ts[:-1]) if len(Ts) > 1 else Ts[0]
    Xva, Tva = Xs[-1], Ts[-1]
    insc = np.ones(NIN, np.float32)
    insc[:9] = 1.0 / Xtr[:, :9].std(dim=0).clamp_min(1e-30).cpu().numpy()
    insc[9] = 1.0 / delta
    outsc = Ttr.std(dim=0).clamp_min(1e-30).cpu().numpy().astype(np.float32)
    mlp = Mlp(seed)
    mlp.set(init_params(seed), np.concatenate([insc, outsc]))
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    nb = Xtr.shape[0] // batch
    t0 = time.time()
    losses = []
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(Xtr.shape[0], device="cuda", generator=g)
        for b in range(nb):
            idx = perm[b * batch:(b + 1) * batch]
            lr_t = lr * 0.5 * (1 + math.cos(math.pi * step / max(1, epochs * nb)))
            want = (b % 200 == 0)
            lv = mlp.train_step(Xtr[idx].contiguous(), Ttr[idx].contiguous(), lr_t, want_loss=want)
            if want:
                losses.append((step, lv))
            step += 1
    torch.cuda.synchronize()
    out["train_seconds"] = time.time() - t0
    out["train_loss"] = losses

    def val_r2(X, T):
        Y = mlp.infer(X)
        r = ((Y - T) ** 2).sum(dim=0) / ((T - T.mean(dim=0)) ** 2).sum(dim=0)
        return [float(1 - v) for v in r.cpu()]

    out["r2_train"] = val_r2(Xtr[: min(Xtr.shape[0], 2_000_000)], Ttr[: min(Xtr.shape[0], 2_000_000)])
    out["r2_validation"] = val_r2(Xva, Tva)
    del Xs, Ts, Xtr, Ttr
    # ---- LES runs -------------------------------------------------------------
    runs = {}
    for name in ("mlp", "dynsmag", "none"):
        s = Solver(cl, dt, xnu, itimescheme=3, precision=_lib.PREC_FP64)
        if name == "mlp":
            check(lib.x3d_solver_set_les_mlp(s.h, mlp.h), "x3d_solver_set_les_mlp")
        elif name == "dynsmag":
            s.set_les(3, 0.15, 0.3)
        s.init_tgv()
        ul = [torch.empty((n_les,) * 3, dtype=torch.float64, device="cuda") for _ in range(3)]
        es = []
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        tstep = 0.0
        for it in range(0, nsteps + 1):
            if it % record_every == 0:
                s.get_velocity_into(*ul)
                es.append(_stats(torch, ul))
            if it < nsteps:
                ev0.record()
                s.step(1)
                ev1.record()
                ev1.synchronize()
                tstep += ev0.elapsed_time(ev1)
        runs[name] = {"E": es, "ms_per_step": tstep / max(1, nsteps)}
        s.close()
    tt = np.array(tdns)
    ef = np.array(edns)

    def diss(e):
        return -np.gradient(np.asarray(e), tt)

    epsf = diss(ef)
    win = tt >= t_train[0]
    out["t"] = tt.tolist()
    out["E_filtered_dns"] = ef.tolist()
    out["eps_filtered_dns"] = epsf.tolist()
    for name, r in runs.items():
        eps = diss(r["E"])
        r["eps"] = eps.tolist()
        r["eps_rel_l2"] = float(np.linalg.norm((eps - epsf)[win]) / np.linalg.norm(epsf[win]))
        r["eps_peak_rel"] = float(abs(eps[win].max() - epsf[win].max()) / epsf[win].max())
        out[name] = r
    out["cost_mlp_over_dynsmag"] = runs["mlp"]["ms_per_step"] / runs["dynsmag"]["ms_per_step"]
    out["params"], out["scales"] = [a.tolist() for a in mlp.get()]
    mlp.close()
    return out
