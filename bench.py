"""Benchmark: Taylor-Green vortex 512^3 incompressible step on GB300.

Metric: grid-points x time-steps per second (Mpts*steps/s) of the full time
step (momentum RHS with 27 compact line solves, AB3 update, divergence,
FFT Poisson solve, gradient, correction), fields resident in HBM.
value = the mixed-precision solver (FP32 operators, FP64 state, time
integration and Poisson FFT); the FP64 solver is reported beside it, together
with the kinetic-energy difference between the two after the same steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--n 512] [--impl ours|reference]
  python bench.py --workload ops [--n 512] [--ops dery,...] [--dtypes f64,f32] [--bcs 0,2]
  python bench.py --workload channel [--steps K] [--warmup W]
  python bench.py --workload les [--steps K] [--warmup W]
  python bench.py --workload les_mlp [--n 512] [--t-end 20] [--out results.json]
  python bench.py --workload freeslip [--steps K] [--warmup W]
  python bench.py --workload mlp [--reps R]

--impl reference times the CPU restatement of the reference's path (the
parity oracle, C++/OpenMP on all host cores) on a bounded sample grid of the
same workload, and reports the same metric.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TGV 512^3 Mpts*steps/s (mixed FP32/FP64 step; FP64 step reported beside it)"
UNIT = "Mpts*steps/s"


# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the fused
# y-line momentum kernel (conv_diff_yz, reads u_j, u_q, a1 and writes out) on
# the 512^3 FP32 fields (ncu --set full capture of
# `bench.py --workload ops --n 512 --ops convdiffy --reps 1`)
CONVDIFF_Y_F32_512_DRAM_BYTES = 1610714112 + 515571200


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(torch, secs, device):
    """The job's time: the slowest rank's (all-reduce MAX over the process
    group; the value itself on one process)."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return secs
    t = torch.tensor([float(secs)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(points_per_rank, steps, ws, secs):
    """Whole-job Mpts*steps/s: the grid points all replicas advanced, over the
    slowest rank's time (weak scaling: every rank runs the full workload)."""
    return points_per_rank * steps * ws / secs / 1e6


class Clocks:
    """Samples nvidia-smi during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_oracle_rate(n=96, steps=3):
    """Oracle TGV AB3 steps on an n^3 sample (all host threads): Mpts*steps/s."""
    import numpy as np
    import oracle
    oracle.build()
    threads = oracle.Oracle.set_threads(os.cpu_count() or 1)
    L = 2 * np.pi
    o = oracle.Oracle(n, n, n, L, L, L)
    x = np.arange(n) * (L / n)
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    ux = np.sin(X) * np.cos(Y) * np.cos(Z)
    uy = -np.cos(X) * np.sin(Y) * np.cos(Z)
    uz = np.zeros_like(ux)
    o.run(ux, uy, uz, 1, 0.002, 1 / 1600.0, 3, 0)  # warm-up
    t0 = time.perf_counter()
    o.run(ux, uy, uz, steps, 0.002, 1 / 1600.0, 3, 0)
    dt = time.perf_counter() - t0
    return n ** 3 * steps / dt / 1e6, threads, dt


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    n = args.ref_n
    rate, threads, dt = cpu_oracle_rate(n, max(1, args.steps // 4))
    sample = "TGV %d^3 AB3 steps (sample of the 512^3 workload; rate per grid point)" % n
    line = {"impl": "reference", "metric": METRIC, "value": round(rate, 4), "unit": UNIT, "n_gpus": args.gpus,
            "steps": max(1, args.steps // 4), "warmup": 1, "ms_per_step": round(1e3 * dt / max(1, args.steps // 4), 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "tgv_%d^3_ab3_cpu_oracle" % n, "grid": [n, n, n], "re": 1600, "dt": 0.002},
            "cpu_baseline": {"value": round(rate, 4), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(rate, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_steps(torch, solver, steps, stream):
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    solver.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def time_kernel(torch, fn, reps, stream):
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def run_ours(args):
    import numpy as np
    import torch
    import incompact3d_gb300 as x3d

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    x3d.build()
    n = args.n
    L = 2 * np.pi
    N = n ** 3
    dt = 0.002
    stream = torch.cuda.current_stream()
    ctx = x3d.Context(n, n, n, L, L, L)
    res = {}
    ke = {}
    solvers = {}
    for prec in (["mixed", "fp64"] if args.precision == "both" else [args.precision]):
        p = x3d.PREC_MIXED if prec == "mixed" else x3d.PREC_FP64
        s = x3d.Solver(ctx, dt, 1 / 1600.0, itimescheme=3, precision=p)
        s.init_tgv()
        s.step(args.warmup)
        torch.cuda.synchronize()
        launches0 = s.lib.x3d_solver_launches_per_step(s.h)
        if ws > 1:
            torch.distributed.barrier()
        with Clocks(local) as clk:
            secs = time_steps(torch, s, args.steps, stream)
        secs = max_over_ranks(torch, secs, "cuda")
        res[prec] = {"secs": secs, "clocks": clk.summary(), "launches": launches0}
        solvers[prec] = s
    # kinetic energy of both solvers after the same number of steps
    if len(solvers) == 2:
        for prec, s in solvers.items():
            ke[prec] = float(s.tgv_stats()[0])
    if args.no_e2e:
        if rank == 0:
            main = res.get("mixed") or res[list(res)[0]]
            print(json.dumps({"metric": METRIC, "value": round(job_rate(N, args.steps, ws, main["secs"]), 3),
                              "unit": UNIT, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": round(1e3 * main["secs"] / args.steps, 3), "partial": "no e2e"}))
        return
    # e2e through the public API with host buffers: H2D velocity (pinned) ->
    # one step -> D2H velocity, every step, on the mixed solver
    e2e = None
    # (the velocity lives in pinned host memory; set/get copy it straight
    # between those buffers and the solver's device state)
    s = solvers.get("mixed") or solvers[list(solvers)[0]]
    host = [torch.empty((n, n, n), dtype=torch.float64, pin_memory=True) for _ in range(3)]
    s.get_velocity_into(*host)
    lib = s.lib
    import ctypes
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    # stream-ordered set / step / get through the public API: each component
    # moves on its own stream, so one component's read-out overlaps another's
    # write-back; the host buffers are complete at the final synchronisation
    e2e_steps = max(1, min(args.steps, 5))
    sp = ctypes.c_void_p(stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        x3d._lib.check(lib.x3d_solver_set_velocity_async(s.h, ptr(host[0]), ptr(host[1]), ptr(host[2]), sp))
        s.step(1)
        x3d._lib.check(lib.x3d_solver_get_velocity_async(s.h, ptr(host[0]), ptr(host[1]), ptr(host[2]), sp))
    x3d._lib.check(lib.x3d_solver_sync(s.h))
    torch.cuda.synchronize()
    e2e_secs = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": round(N / e2e_secs / 1e6 * ws, 3), "unit": UNIT, "h2d_bytes_per_step": 3 * N * 8,
           "d2h_bytes_per_step": 3 * N * 8}
    del host
    # dominant kernel by launch-list share, timed alone with CUDA events: the
    # fused y-line momentum kernel on 512^3 FP32 fields (algorithmic bytes:
    # read u_j, u_q, a1, write out = 4 N * 4)
    uj32 = torch.randn((n, n, n), dtype=torch.float32, device="cuda")
    uq32 = torch.randn((n, n, n), dtype=torch.float32, device="cuda")
    a132 = torch.randn((n, n, n), dtype=torch.float32, device="cuda")
    o32 = torch.empty_like(uq32)
    ksec = time_kernel(torch, lambda: ctx.conv_diff(1, 0, uj32, uq32, a132, 1 / 1600.0, out=o32), 20, stream)
    kbytes = 4 * N * 4
    del uj32, uq32, a132, o32
    u64 = torch.randn((n, n, n), dtype=torch.float64, device="cuda")
    o64 = torch.empty_like(u64)
    ksec64 = time_kernel(torch, lambda: ctx.apply(1, x3d.OP_DER1, 0, u64, out=o64), 10, stream)
    pk, pk_kind = peaks()
    if rank != 0:
        return
    main = res.get("mixed") or res[list(res)[0]]
    secs = main["secs"]
    value = job_rate(N, args.steps, ws, secs)
    cpu_rate, cpu_threads, _ = cpu_oracle_rate(args.cpu_n, 1) if not args.no_cpu else (None, 0, 0)
    achieved = kbytes / ksec / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "mixed f32/f64" if "mixed" in res else "f64",
        "data": "synthetic",
        "config": {"workload": "tgv_512^3_ab3" if n == 512 else "tgv_%d^3_ab3" % n, "grid": [n, n, n],
                   "re": 1600, "dt": dt, "time_scheme": "AB3", "l2": "inputs larger than L2 (fields %.2f GB)"
                   % (N * 8 / 1e9), "parallelism": "replicas" if ws > 1 else "1gpu"},
        "clocks": main["clocks"],
        "e2e": e2e,
        "gpu_launches": int(main["launches"] * args.steps),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk, "unit": "GB/s",
                     "frac": round(achieved / pk, 4),
                     "traffic": CONVDIFF_Y_F32_512_DRAM_BYTES if n == 512 else None,
                     "kernel": "conv_diff_yz (fused y-line momentum RHS, 3 compact solves, FP32) 512^3",
                     "peak_source": pk_kind},
        "cpu_baseline": {"value": round(cpu_rate, 4) if cpu_rate else None, "unit": UNIT, "cores": cpu_threads,
                         "kind": "port",
                         "sample": "oracle TGV %d^3, 1 AB3 step, rate per grid point" % args.cpu_n},
    }
    if "fp64" in res:
        f = res["fp64"]
        line["fp64"] = {"value": round(N * args.steps * ws / f["secs"] / 1e6, 3),
                        "ms_per_step": round(1e3 * f["secs"] / args.steps, 3), "clocks": f["clocks"],
                        "dery_f64_gbs": round(2 * N * 8 / ksec64 / 1e9, 1)}
    if ke:
        line["ke_mixed_minus_fp64"] = ke["mixed"] - ke["fp64"]
        line["ke_fp64"] = ke["fp64"]
    print(json.dumps(line), flush=True)


def spectral_field(torch, n, L, periodic, seed=20261204, nmodes=64, kmax=32, zero_mean=False):
    """Operator-microbench input on the device, shape (n, n, n), FP64:
    f = sum_m A_m cos(k_m . x + phi_m), integer k_m with 1 <= |k| <= kmax
    (components in [-kmax, kmax]), A_m = |k|^(-5/3) / sqrt(sum |k|^(-10/3)),
    phi_m ~ U[0, 2pi); k drawn first, then the phases."""
    import numpy as np
    rng = np.random.default_rng(seed)
    ks = []
    while len(ks) < nmodes:
        k = rng.integers(-kmax, kmax + 1, size=3)
        r = float(np.sqrt((k * k).sum()))
        if 1 <= r <= kmax:
            ks.append(k)
    ph = rng.uniform(0, 2 * np.pi, size=nmodes)
    amp = np.array([float(np.sqrt((k * k).sum())) ** (-5 / 3) for k in ks])
    amp /= np.sqrt((amp ** 2).sum())
    d = L / n if periodic else L / (n - 1)
    x = torch.arange(n, dtype=torch.float64, device="cuda") * d
    f = torch.zeros((n, n, n), dtype=torch.float64, device="cuda")
    for k, a, p in zip(ks, amp, ph):
        # k . x for the (z, y, x) index order
        arg = (k[2] * x)[:, None, None] + (k[1] * x)[None, :, None] + (k[0] * x)[None, None, :] + p
        f += a * torch.cos(arg)
    if zero_mean:
        f -= f.mean()
    return f


def run_ops(args):
    """Operator microbench: compact first/second derivatives and the filter
    along x, y and z on n^3 fields, FP64 and FP32, periodic (ncl=0) and
    Dirichlet (ncl=2) boundaries, plus the FFT Poisson solve on a zero-mean
    RHS; one JSON line per case with GB/s against the HBM peak (algorithmic
    bytes (N_in + N_out) * element size; inputs larger than L2)."""
    import numpy as np
    import torch
    import incompact3d_gb300 as x3d

    x3d.build()
    n = args.n
    L = 2 * np.pi
    N = n ** 3
    stream = torch.cuda.current_stream()
    pk, pk_kind = peaks()
    want = set(args.ops.split(",")) if args.ops else None
    names = {(x3d.OP_DER1, 0): "derx", (x3d.OP_DER1, 1): "dery", (x3d.OP_DER1, 2): "derz",
             (x3d.OP_DER2, 0): "derxx", (x3d.OP_DER2, 1): "deryy", (x3d.OP_DER2, 2): "derzz",
             (x3d.OP_FIL, 0): "filx", (x3d.OP_FIL, 1): "fily", (x3d.OP_FIL, 2): "filz"}
    for bc in [int(b) for b in args.bcs.split(",")]:
        ctx = x3d.Context(n, n, n, L, L, L, bc=((bc, bc),) * 3)
        f64 = spectral_field(torch, n, L, bc == 0)
        for dt in args.dtypes.split(","):
            u = f64 if dt == "f64" else f64.float()
            o = torch.empty_like(u)
            es = u.element_size()
            for (op, axis), nm in names.items():
                if want and nm not in want:
                    continue
                npaire = 1 if op == x3d.OP_DER2 or op == x3d.OP_FIL else 0
                sec = time_kernel(torch, lambda: ctx.apply(axis, op, npaire, u, out=o), args.reps, stream)
                gbs = 2 * N * es / sec / 1e9
                print(json.dumps({"op": nm, "dtype": dt, "ncl": bc, "n": n, "ms": round(1e3 * sec, 4),
                                  "gbs": round(gbs, 1), "frac": round(gbs / pk, 4), "peak_source": pk_kind}),
                      flush=True)
            del u, o
        del ctx, f64
    cd = [a for a in ("convdiffx", "convdiffy", "convdiffz") if want is None or a in want]
    if cd:
        # fused momentum term of one direction (FP32, periodic): reads u_j,
        # u_q and the running sum, writes the result -> 4 N * 4 bytes
        ctx = x3d.Context(n, n, n, L, L, L)
        uj = spectral_field(torch, n, L, True, seed=1).float()
        uq = spectral_field(torch, n, L, True, seed=2).float()
        a1 = spectral_field(torch, n, L, True, seed=3).float()
        o = torch.empty_like(uq)
        for nm in cd:
            axis = "xyz".index(nm[-1])
            sec = time_kernel(torch, lambda: ctx.conv_diff(axis, 1, uj, uq, a1, 1 / 1600.0, out=o), args.reps,
                              stream)
            gbs = 4 * N * 4 / sec / 1e9
            print(json.dumps({"op": nm, "dtype": "f32", "ncl": 0, "n": n, "ms": round(1e3 * sec, 4),
                              "gbs": round(gbs, 1), "frac": round(gbs / pk, 4), "peak_source": pk_kind}),
                  flush=True)
        del ctx, uj, uq, a1, o
    if want is None or "poisson" in want:
        ctx = x3d.Context(n, n, n, L, L, L)
        rhs0 = spectral_field(torch, n, L, True, zero_mean=True)
        rhs = torch.empty_like(rhs0)
        arith = set(args.poisson_arith.split(","))
        for prec, nm in ((0, "fp64"), (2, "double-float"), (1, "fp32")):
            if nm not in arith:
                continue
            def solve():
                rhs.copy_(rhs0)
                ctx.poisson(rhs, precision=prec)
            copy_sec = time_kernel(torch, lambda: rhs.copy_(rhs0), args.reps, stream)
            sec = time_kernel(torch, solve, args.reps, stream) - copy_sec
            gbs = 2 * N * 8 / sec / 1e9
            print(json.dumps({"op": "poisson_000", "arith": nm, "n": n, "ms": round(1e3 * sec, 4),
                              "gbs": round(gbs, 1), "frac": round(gbs / pk, 4), "peak_source": pk_kind}),
                  flush=True)


CHANNEL_L = (8 * 3.141592653589793, 2.0, 3 * 3.141592653589793)
CHANNEL_BETA = 0.259065151


def channel_ic(np, nx, ny, nz, yp, Ly=2.0, noise=0.125, seed=20261204):
    """Laminar Poiseuille profile plus modulated uniform noise (seeded PCG64)."""
    rng = np.random.default_rng(seed)
    y = yp - Ly / 2
    um = np.exp(-0.2 * y * y)
    r = [rng.uniform(size=(nz, ny, nx)) for _ in range(3)]
    ux = noise * um[None, :, None] * (2 * r[0] - 1) + (1 - y * y)[None, :, None]
    uy = noise * um[None, :, None] * (2 * r[1] - 1)
    uz = noise * um[None, :, None] * (2 * r[2] - 1)
    return ux, uy, uz


def run_channel(args):
    """Turbulent channel, FP64: 256x129x128 on 8pi x 2 x 3pi, y stretched at both
    walls (istret=2, beta=0.259), constant flow rate, RK3, dt=0.002, Re=4200.
    One JSON line: Mpts*steps/s of the GPU solver, with the CPU oracle timed
    on a sample grid beside it."""
    import numpy as np
    import torch
    import incompact3d_gb300 as x3d

    x3d.build()
    nx, ny, nz = 256, 129, 128
    bc = ((0, 0), (2, 2), (0, 0))
    ctx = x3d.Context(nx, ny, nz, *CHANNEL_L, bc=bc, istret=2, beta=CHANNEL_BETA)
    s = x3d.Solver(ctx, 0.002, 1 / 4200.0, itimescheme=5, precision=x3d.PREC_FP64)
    s.set_channel()
    s.set_velocity(*channel_ic(np, nx, ny, nz, ctx.stretching()["yp"]))
    s.step(args.warmup)
    stream = torch.cuda.current_stream()
    with Clocks(0) as clk:
        secs = time_steps(torch, s, args.steps, stream)
    N = nx * ny * nz
    ub = s.bulk_velocity()
    line = {"workload": "channel_256x129x128_rk3_fp64", "metric": "channel Mpts*steps/s", "unit": UNIT,
            "value": round(N * args.steps / secs / 1e6, 3), "ms_per_step": round(1e3 * secs / args.steps, 3),
            "steps": args.steps, "warmup": args.warmup, "dtype": "f64", "clocks": clk.summary(),
            "launches_per_step": s.lib.x3d_solver_launches_per_step(s.h), "bulk_velocity": float(ub[-1]),
            "divmax": s.divmax()}
    if not args.no_cpu:
        import oracle
        oracle.build()
        threads = oracle.Oracle.set_threads(os.cpu_count() or 1)
        m = (64, 65, 32)
        o = oracle.Oracle(*m, *CHANNEL_L, bc=bc, istret=2, beta=CHANNEL_BETA)
        ic = channel_ic(np, *m, o.stretching()["yp"])
        o.run_channel(*ic, 1, 0.002, 1 / 4200.0, itimescheme=5)
        t0 = time.perf_counter()
        o.run_channel(*ic, 2, 0.002, 1 / 4200.0, itimescheme=5)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": round(m[0] * m[1] * m[2] * 2 / dt / 1e6, 4), "unit": UNIT,
                                "cores": threads, "kind": "port",
                                "sample": "oracle channel 64x65x32, 2 RK3 steps, rate per grid point"}
    print(json.dumps(line), flush=True)


def run_les(args):
    """LES of the TGV at Re=5000 on 128^3 (FP64, AB3, dt=0.005): the
    dynamic-Smagorinsky step and the Smagorinsky step timed beside the plain
    (no-model) step; the ratio is the SGS model's cost factor."""
    import numpy as np
    import torch
    import incompact3d_gb300 as x3d

    x3d.build()
    n = 128
    L = 2 * np.pi
    ctx = x3d.Context(n, n, n, L, L, L)
    stream = torch.cuda.current_stream()
    out = {"workload": "tgv_les_128^3_re5000_ab3_fp64", "metric": "LES step Mpts*steps/s", "unit": UNIT,
           "dtype": "f64", "steps": args.steps, "warmup": args.warmup}
    for name, jles in (("plain", 0), ("smag", 1), ("dynsmag", 3)):
        s = x3d.Solver(ctx, 0.005, 1 / 5000.0, itimescheme=3, precision=x3d.PREC_FP64)
        if jles:
            s.set_les(jles, 0.14, 0.3)
        s.init_tgv()
        s.step(args.warmup)
        secs = time_steps(torch, s, args.steps, stream)
        out[name] = {"ms_per_step": round(1e3 * secs / args.steps, 3),
                     "value": round(n ** 3 * args.steps / secs / 1e6, 3),
                     "launches_per_step": s.lib.x3d_solver_launches_per_step(s.h)}
        s.close()
    # the learned closure (untrained weights: the cost does not depend on them),
    # inference on FP32 CUDA cores and on the tensor cores (tcgen05, BF16 split)
    from incompact3d_gb300 import sgs
    m = sgs.Mlp(seed=0)
    for name, tc in (("mlp", False), ("mlp_tc", True)):
        m.set_tensor_cores(tc)
        s = x3d.Solver(ctx, 0.005, 1 / 5000.0, itimescheme=3, precision=x3d.PREC_FP64)
        s.init_tgv()
        x3d._lib.check(s.lib.x3d_solver_set_les_mlp(s.h, m.h), "x3d_solver_set_les_mlp")
        s.step(args.warmup)
        secs = time_steps(torch, s, args.steps, stream)
        out[name] = {"ms_per_step": round(1e3 * secs / args.steps, 3),
                     "value": round(n ** 3 * args.steps / secs / 1e6, 3),
                     "launches_per_step": s.lib.x3d_solver_launches_per_step(s.h)}
        s.close()
    out.update(mlp_infer_times(torch, m, n ** 3, 20))
    m.close()
    out["value"] = out["dynsmag"]["value"]
    out["dynsmag_over_plain"] = round(out["dynsmag"]["ms_per_step"] / out["plain"]["ms_per_step"], 3)
    out["mlp_tc_over_dynsmag"] = round(out["mlp_tc"]["ms_per_step"] / out["dynsmag"]["ms_per_step"], 3)
    print(json.dumps(out), flush=True)


def mlp_infer_times(torch, m, npts, reps):
    """CUDA-event time of the closure's inference on npts feature rows, FP32
    CUDA-core kernel and tensor-core kernel; network flops = 2 (10*64 + 64*64
    + 64*6) per point (the tensor-core kernel issues 3x that as split MMAs)."""
    stream = torch.cuda.current_stream()
    X = torch.randn((npts, 10), dtype=torch.float32, device="cuda")
    flop = 2.0 * npts * (10 * 64 + 64 * 64 + 64 * 6)
    out = {}
    for name, tc in (("infer_fp32", False), ("infer_tc", True)):
        m.set_tensor_cores(tc)
        for _ in range(3):
            m.infer(X)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            m.infer(X)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"points": npts, "ms": round(ms, 4), "tflops_network": round(flop / ms / 1e9, 2)}
    m.status()
    return out


def run_mlp(args):
    """Inference of the learned closure alone on 128^3 feature rows."""
    import torch
    import incompact3d_gb300 as x3d
    from incompact3d_gb300 import sgs

    x3d.build()
    m = sgs.Mlp(seed=0)
    out = {"workload": "sgs_mlp_inference_128^3", "unit": "ms"}
    out.update(mlp_infer_times(torch, m, 128 ** 3, args.reps))
    m.close()
    print(json.dumps(out), flush=True)


def run_freeslip(args):
    """The reference's own regression case (tests/TGV-Taylor-Green-vortex):
    TGV in the free-slip box [0, pi]^3 with 65^3 nodes, Re = 1600, RK3,
    dt = 0.005, FP64 (poisson_11x); the statistics row after the timed steps
    is printed beside the rate for a diff against reference_time_evol.dat."""
    import numpy as np
    import torch
    import incompact3d_gb300 as x3d

    x3d.build()
    n, L, dt = 65, np.pi, 0.005
    ctx = x3d.Context(n, n, n, L, L, L, bc=((1, 1), (1, 1), (1, 1)))
    s = x3d.Solver(ctx, dt, 1 / 1600.0, itimescheme=5, precision=x3d.PREC_FP64)
    x = np.arange(n) * (L / (n - 1))
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    s.set_velocity(np.sin(X) * np.cos(Y) * np.cos(Z), -np.cos(X) * np.sin(Y) * np.cos(Z), np.zeros((n, n, n)))
    stream = torch.cuda.current_stream()
    s.step(args.warmup)
    secs = time_steps(torch, s, args.steps, stream)
    itime = args.warmup + args.steps
    st = s.tgv_stats()
    out = {"workload": "tgv_freeslip_65^3_rk3_fp64", "metric": "free-slip TGV Mpts*steps/s", "unit": UNIT,
           "value": round(n ** 3 * args.steps / secs / 1e6, 3), "ms_per_step": round(1e3 * secs / args.steps, 3),
           "steps": args.steps, "warmup": args.warmup, "dtype": "f64",
           "launches_per_step": s.lib.x3d_solver_launches_per_step(s.h),
           "stats_row": [(itime - 1) * dt] + [float(v) for v in st]}
    s.close()
    if not args.no_cpu:
        out["cpu_baseline"] = freeslip_cpu_baseline(np, n, L, dt)
    print(json.dumps(out), flush=True)


def freeslip_cpu_baseline(np, n, L, dt, steps=4):
    """The oracle on the same free-slip case (RK3, FP64) on all host cores."""
    import oracle
    oracle.build()
    threads = oracle.Oracle.set_threads(os.cpu_count() or 1)
    o = oracle.Oracle(n, n, n, L, L, L, bc=((1, 1), (1, 1), (1, 1)))
    x = np.arange(n) * (L / (n - 1))
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    ic = (np.sin(X) * np.cos(Y) * np.cos(Z), -np.cos(X) * np.sin(Y) * np.cos(Z), np.zeros((n, n, n)))
    o.run(*ic, 1, dt, 1 / 1600.0, itimescheme=5, every=1)
    t0 = time.perf_counter()
    o.run(*ic, steps, dt, 1 / 1600.0, itimescheme=5, every=steps)
    sec = time.perf_counter() - t0
    return {"value": round(n ** 3 * steps / sec / 1e6, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle on the same {n}^3 free-slip case, {steps} RK3 steps"}


def run_les_mlp(args):
    """Learned SGS closure pipeline: TGV DNS at Re=5000 (n^3, mixed solver,
    dt = 0.001; dt = 0.002 diverged near t = 7.3 at 512^3 with AB3) ->
    box-filtered (ratio 4) training snapshots at t = 2..10 -> MLP training ->
    LES to t = 20 on the /4 grid with the MLP, dynamic Smagorinsky and no
    model; dissipation errors against the filtered DNS and the step cost ratio."""
    import incompact3d_gb300 as x3d
    from incompact3d_gb300 import sgs

    x3d.build()
    n = args.n
    r = sgs.run_pipeline(n_dns=n, n_les=n // 4, re=5000.0, dt=0.002, dt_dns=0.001, t_end=args.t_end,
                         t_train=(2.0, 10.0), snap_every=1.0, epochs=args.epochs, batch=16384, record_every=10,
                         flux_lambda=args.flux_lambda, data_in=args.data_in or None,
                         data_out=args.data_out or None)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(r, f)
    line = {"workload": "tgv_les_mlp_%d^3_dns_%d^3_les_re5000" % (n, n // 4), "metric": "LES dissipation error vs "
            "filtered DNS", "unit": "relative L2 over t in [2, t_end]", "t_end": args.t_end,
            "mlp": {k: r["mlp"][k] for k in ("eps_rel_l2", "eps_peak_rel", "ms_per_step")},
            "dynsmag": {k: r["dynsmag"][k] for k in ("eps_rel_l2", "eps_peak_rel", "ms_per_step")},
            "none": {k: r["none"][k] for k in ("eps_rel_l2", "eps_peak_rel", "ms_per_step")},
            "cost_mlp_over_dynsmag": r["cost_mlp_over_dynsmag"], "r2_validation": r["r2_validation"],
            "flux_ratio_validation": r["flux_ratio_validation"], "flux_lambda": r["flux_lambda"],
            "dns_seconds": r["dns_seconds"], "train_seconds": r["train_seconds"]}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="tgv", choices=["tgv", "ops", "channel", "les", "les_mlp", "freeslip", "mlp"],
                    help="tgv: the time-step benchmark (default); ops: operator microbench lines; "
                         "channel: the stretched turbulent channel (FP64)")
    ap.add_argument("--ops", default="", help="ops workload: comma list (derx,...,filz,poisson)")
    ap.add_argument("--dtypes", default="f64,f32")
    ap.add_argument("--bcs", default="0,2")
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--poisson-arith", default="fp64,double-float,fp32")
    ap.add_argument("--t-end", type=float, default=20.0)
    ap.add_argument("--out", default="")
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--flux-lambda", type=float, default=1.0)
    ap.add_argument("--data-in", default="")
    ap.add_argument("--data-out", default="")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="both", choices=["both", "mixed", "fp64"])
    ap.add_argument("--cpu-n", type=int, default=64)
    ap.add_argument("--ref-n", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="profiling runs: time the step loop only (no e2e, kernel or CPU legs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "ops":
        run_ops(args)
    elif args.workload == "channel":
        run_channel(args)
    elif args.workload == "freeslip":
        run_freeslip(args)
    elif args.workload == "mlp":
        run_mlp(args)
    elif args.workload == "les":
        run_les(args)
    elif args.workload == "les_mlp":
        run_les_mlp(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
