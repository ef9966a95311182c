"""Learned subgrid-stress closure for the TGV LES (FP32 MLP on the GPU).

The model maps the 9 resolved velocity gradients du_i/dx_j and the filter
width to the 6 subgrid stresses tau_ij; it is trained on box-filtered (ratio
4) snapshots of a DNS run by this package's own solver and then used inside
the LES time step (``Solver.set_les_mlp``).  The dynamic Smagorinsky model of
the reference (src/les_models.f90:333-903) is the fallback and the cost
baseline, and the model's error is measured against the box-filtered DNS.

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

    def set_flux_loss(self, lam, pscale):
        """Add lam * ((Pi_model - Pi_data) / pscale)^2 to the training loss,
        Pi = tau_ij S_ij the subgrid energy flux of a sample."""
        check(self.lib.x3d_mlp_set_flux_loss(self.h, ctypes.c_float(lam), ctypes.c_float(pscale)),
              "x3d_mlp_set_flux_loss")

    def set_tensor_cores(self, on=True):
        """Run inference (x3d_mlp_infer and the solver's closure) as tcgen05
        MMAs with BF16 hi / lo split operands instead of FP32 CUDA cores."""
        check(self.lib.x3d_mlp_set_tensor_cores(self.h, 1 if on else 0), "x3d_mlp_set_tensor_cores")

    def status(self):
        """Raises if a bounded wait inside a tensor-core inference ran out."""
        check(self.lib.x3d_mlp_status(self.h), "x3d_mlp_status")

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


def dns_dataset(n_dns=512, n_les=128, re=5000.0, dt=0.002, dt_dns=None, t_end=20.0, t_train=(2.0, 10.0),
                snap_every=1.0, record_every=10):
    """Run the DNS (mixed-precision solver) and return the box-filtered data:
    training snapshots (all but the last) and validation snapshot (the last)
    as feature / target arrays on the device, and the filtered kinetic energy
    history at every record_every LES steps."""
    torch = _torch()
    L = 2 * math.pi
    xnu = 1.0 / re
    lib = _lib.load()
    dt_dns = dt if dt_dns is None else dt_dns
    sub = int(round(dt / dt_dns))
    cd = Context(n_dns, n_dns, n_dns, L, L, L)
    cl = Context(n_les, n_les, n_les, L, L, L)
    sd = Solver(cd, dt_dns, xnu, itimescheme=3, precision=_lib.PREC_MIXED)
    sd.init_tgv()
    u = [torch.empty((n_dns,) * 3, dtype=torch.float64, device="cuda") for _ in range(3)]
    nsteps = int(round(t_end / dt))
    snaps = set(int(round(t / dt)) for t in np.arange(t_train[0], t_train[1] + 1e-9, snap_every))
    Xs, Ts, tdns, edns = [], [], [], []
    delta = None
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
            sd.step(sub)
    torch.cuda.synchronize()
    secs = time.time() - t0
    sd.close()
    if not all(np.isfinite(edns)):
        raise FloatingPointError("the DNS diverged (filtered kinetic energy not finite)")
    return {"Xtr": torch.cat(Xs[:-1]), "Ttr": torch.cat(Ts[:-1]), "Xva": Xs[-1], "Tva": Ts[-1], "delta": delta,
            "t": np.array(tdns), "E": np.array(edns), "dns_seconds": secs}


def save_dataset(path, d, ntrain=400_000, nval=100_000, seed=0):
    """A random subsample of the box-filtered data (features, targets) and the
    filtered kinetic-energy history, as an .npz file."""
    torch = _torch()
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    it = torch.randperm(d["Xtr"].shape[0], device="cuda", generator=g)[:ntrain]
    iv = torch.randperm(d["Xva"].shape[0], device="cuda", generator=g)[:nval]
    np.savez(path, Xtr=d["Xtr"][it].cpu().numpy(), Ttr=d["Ttr"][it].cpu().numpy(), Xva=d["Xva"][iv].cpu().numpy(),
             Tva=d["Tva"][iv].cpu().numpy(), delta=d["delta"], t=d["t"], E=d["E"])


def load_dataset(path):
    torch = _torch()
    z = np.load(path)
    return {"Xtr": torch.from_numpy(z["Xtr"]).cuda(), "Ttr": torch.from_numpy(z["Ttr"]).cuda(),
            "Xva": torch.from_numpy(z["Xva"]).cuda(), "Tva": torch.from_numpy(z["Tva"]).cuda(),
            "delta": float(z["delta"]), "t": z["t"], "E": z["E"], "dns_seconds": 0.0}


def flux(X, T):
    """Subgrid energy flux tau_ij S_ij of samples (raw gradient features)."""
    S = [X[:, 0], X[:, 4], X[:, 8], 0.5 * (X[:, 1] + X[:, 3]), 0.5 * (X[:, 2] + X[:, 6]), 0.5 * (X[:, 5] + X[:, 7])]
    w = [1.0, 1.0, 1.0, 2.0, 2.0, 2.0]
    return sum(w[m] * T[:, m] * S[m] for m in range(6))


def train(d, epochs=3, batch=16384, lr=1e-3, flux_lambda=1.0, seed=0):
    """Train the MLP on the dataset; returns (model, log dict)."""
    torch = _torch()
    Xtr, Ttr = d["Xtr"], d["Ttr"]
    insc = np.ones(NIN, np.float32)
    insc[:9] = 1.0 / Xtr[:, :9].std(dim=0).clamp_min(1e-30).cpu().numpy()
    insc[9] = 1.0 / d["delta"]
    outsc = Ttr.std(dim=0).clamp_min(1e-30).cpu().numpy().astype(np.float32)
    mlp = Mlp(seed)
    mlp.set(init_params(seed), np.concatenate([insc, outsc]))
    pscale = float(flux(Xtr, Ttr).std())
    mlp.set_flux_loss(flux_lambda, pscale)
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

    def r2(X, T):
        Y = mlp.infer(X)
        r = ((Y - T) ** 2).sum(dim=0) / ((T - T.mean(dim=0)) ** 2).sum(dim=0)
        pf, tf = flux(X, Y), flux(X, T)
        return [float(1 - v) for v in r.cpu()], float(pf.mean() / tf.mean())

    m = min(Xtr.shape[0], 2_000_000)
    r2t, ft = r2(Xtr[:m], Ttr[:m])
    r2v, fv = r2(d["Xva"], d["Tva"])
    return mlp, {"train_seconds": time.time() - t0, "train_loss": losses, "r2_train": r2t, "r2_validation": r2v,
                 "flux_ratio_train": ft, "flux_ratio_validation": fv, "flux_lambda": flux_lambda}


def les_compare(mlp, d, n_les=128, re=5000.0, dt=0.002, t_end=20.0, t_from=2.0, record_every=10):
    """LES runs (MLP, dynamic Smagorinsky, no model) against the filtered DNS."""
    torch = _torch()
    L = 2 * math.pi
    xnu = 1.0 / re
    lib = _lib.load()
    cl = Context(n_les, n_les, n_les, L, L, L)
    nsteps = int(round(t_end / dt))
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
    tt = np.asarray(d["t"])
    ef = np.asarray(d["E"])

    def diss(e):
        return -np.gradient(np.asarray(e), tt)

    epsf = diss(ef)
    win = tt >= t_from
    out = {"t": tt.tolist(), "E_filtered_dns": ef.tolist(), "eps_filtered_dns": epsf.tolist()}
    for name, r in runs.items():
        eps = diss(r["E"])
        r["eps"] = eps.tolist()
        r["eps_rel_l2"] = float(np.linalg.norm((eps - epsf)[win]) / np.linalg.norm(epsf[win]))
        r["eps_peak_rel"] = float(abs(eps[win].max() - epsf[win].max()) / epsf[win].max())
        out[name] = r
    out["cost_mlp_over_dynsmag"] = runs["mlp"]["ms_per_step"] / runs["dynsmag"]["ms_per_step"]
    return out


def run_pipeline(n_dns=512, n_les=128, re=5000.0, dt=0.002, dt_dns=None, t_end=20.0, t_train=(2.0, 10.0),
                 snap_every=1.0, epochs=3, batch=16384, lr=1e-3, flux_lambda=1.0, record_every=10, seed=0,
                 data_in=None, data_out=None):
    """DNS -> box-filtered training set -> MLP training -> LES comparison.
    data_in: load a saved dataset instead of running the DNS; data_out: save a
    subsample of the DNS data for later runs."""
    if data_in:
        d = load_dataset(data_in)
    else:
        d = dns_dataset(n_dns, n_les, re, dt, dt_dns, t_end, t_train, snap_every, record_every)
        if data_out:
            save_dataset(data_out, d, seed=seed)
    mlp, log = train(d, epochs, batch, lr, flux_lambda, seed)
    out = {"n_dns": n_dns, "n_les": n_les, "re": re, "dt": dt, "dt_dns": dt_dns, "t_end": t_end,
           "dns_seconds": d["dns_seconds"]}
    out.update(log)
    out.update(les_compare(mlp, d, n_les, re, dt, t_end, t_train[0], record_every))
    out["params"], out["scales"] = [a.tolist() for a in mlp.get()]
    mlp.close()
    return out
