"""Taylor-Green vortex on the GPU solver vs the CPU oracle.

Configuration: 64^3 triply periodic on [0,2pi]^3, Re=1600, AB3 (Euler and AB2
start-up, src/time_integrators.f90:86-100), dt=0.005, 200 steps, statistics of
postprocess_tgv (src/Case-TGV.f90:189-477) every 10 steps.  FP64 must match the
oracle within 1e-10 (relative); the mixed-precision solver must keep the
kinetic energy within 1e-6 of the FP64 run.
"""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu
L = 2 * np.pi


def tgv_ic(n):
    x = np.arange(n) * (L / n)
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    ux = np.sin(X) * np.cos(Y) * np.cos(Z)
    uy = -np.cos(X) * np.sin(Y) * np.cos(Z)
    return ux, uy, np.zeros_like(ux)


def run_gpu(gpu_lib, n, nsteps, dt, itimescheme, precision, every=10):
    ctx = gpu_lib.Context(n, n, n, L, L, L)
    s = gpu_lib.Solver(ctx, dt, 1 / 1600.0, itimescheme=itimescheme, precision=precision)
    s.set_velocity(*tgv_ic(n))
    rows = []
    for it in range(1, nsteps + 1):
        s.step(1)
        if it % every == 0:
            rows.append([(it - 1) * dt, *s.tgv_stats()])
    return np.array(rows), s, ctx


@pytest.fixture(scope="module")
def oracle_tgv64(oracle_mod):
    o = oracle_mod.Oracle(64, 64, 64, L, L, L)
    ux, uy, uz = tgv_ic(64)
    a, b, c, rows, dmax = o.run(ux, uy, uz, 200, 0.005, 1 / 1600.0, 3, 10)
    return rows, (a, b, c), dmax


def test_tgv64_ab3_fp64_matches_oracle(gpu_lib, oracle_tgv64):
    rows_o, u_o, dmax_o = oracle_tgv64
    rows, s, ctx = run_gpu(gpu_lib, 64, 200, 0.005, 3, gpu_lib.PREC_FP64)
    assert rows.shape == rows_o.shape == (20, 5)
    for col, name in ((1, "E_k"), (2, "eps"), (3, "eps2"), (4, "enstrophy")):
        err = np.max(np.abs(rows[:, col] - rows_o[:, col]) / np.abs(rows_o[:, col]))
        assert err < 1e-10, (name, err)
    u = s.get_velocity()
    for a, b in zip(u, u_o):
        assert relerr(a, b) < 1e-10
    assert s.divmax() < 1e-12


def test_tgv64_mixed_precision_energy(gpu_lib, oracle_tgv64):
    rows_o, _, _ = oracle_tgv64
    rows, s, ctx = run_gpu(gpu_lib, 64, 200, 0.005, 3, gpu_lib.PREC_MIXED)
    ke_err = np.max(np.abs(rows[:, 1] - rows_o[:, 1]))
    assert ke_err < 1e-6, ke_err
    # divergence and gradient run in FP32 in this mode: the projection is exact
    # to binary32 round-off of the staggered operators, not to FP64's.
    assert s.divmax() < 1e-3


def test_tgv_rk3_matches_oracle(oracle_mod, gpu_lib):
    n = 32
    o = oracle_mod.Oracle(n, n, n, L, L, L)
    ux, uy, uz = tgv_ic(n)
    _, _, _, rows_o, _ = o.run(ux, uy, uz, 20, 0.01, 1 / 1600.0, 5, 10)
    rows, s, ctx = run_gpu(gpu_lib, n, 20, 0.01, 5, gpu_lib.PREC_FP64)
    assert np.max(np.abs(rows[:, 1:] - rows_o[:, 1:]) / np.abs(rows_o[:, 1:])) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pinned_host_transfer_matches_pageable(gpu_lib, precision):
    """set/get with page-locked host buffers (read and written by kernels
    directly) give the same velocity, bit for bit, as pageable numpy buffers."""
    torch = pytest.importorskip("torch")
    n = 32
    ctx = gpu_lib.Context(n, n, n, L, L, L)
    ic = tgv_ic(n)
    res = []
    for pinned in (False, True):
        prec = gpu_lib.PREC_FP64 if precision == "fp64" else gpu_lib.PREC_MIXED
        s = gpu_lib.Solver(ctx, 0.005, 1 / 1600.0, itimescheme=3, precision=prec)
        if pinned:
            h = [torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for v in ic]
            s.set_velocity(*h)
        else:
            s.set_velocity(*ic)
        s.step(3)
        if pinned:
            out = [torch.empty((n, n, n), dtype=torch.float64).pin_memory() for _ in range(3)]
            s.get_velocity_into(*out)
            out = [o.numpy() for o in out]
        else:
            out = s.get_velocity()
        res.append(out)
    for a, b in zip(*res):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_round_trip_matches_device_loop(gpu_lib, precision):
    """set / step / get through pinned host buffers with the stream-ordered
    calls, against the device-resident run (time level and history kept).  The
    FP64 state round-trips exactly: bit for bit.  The mixed solver's
    double-float state round-trips its binary64 value exactly but is re-split
    into the canonical hi / lo pair, so its binary32 operand can differ in the
    last bit: 1e-10 of the largest value after 6 steps."""
    import ctypes
    import torch
    n = 64
    prec = gpu_lib.PREC_FP64 if precision == "fp64" else gpu_lib.PREC_MIXED
    ctx = gpu_lib.Context(n, n, n, L, L, L)
    a = gpu_lib.Solver(ctx, 0.005, 1.0 / 1600.0, itimescheme=3, precision=prec)
    b = gpu_lib.Solver(ctx, 0.005, 1.0 / 1600.0, itimescheme=3, precision=prec)
    a.init_tgv()
    b.init_tgv()
    host = [torch.empty((n, n, n), dtype=torch.float64, pin_memory=True) for _ in range(3)]
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib = b.lib
    lib.x3d_solver_get_velocity_async(b.h, ptr(host[0]), ptr(host[1]), ptr(host[2]), sp)
    for _ in range(6):
        a.step(1)
        assert lib.x3d_solver_set_velocity_async(b.h, ptr(host[0]), ptr(host[1]), ptr(host[2]), sp) == 0
        b.step(1)
        assert lib.x3d_solver_get_velocity_async(b.h, ptr(host[0]), ptr(host[1]), ptr(host[2]), sp) == 0
    assert lib.x3d_solver_sync(b.h) == 0
    ref = [torch.from_numpy(v) for v in a.get_velocity()]
    for h, r in zip(host, ref):
        if precision == "fp64":
            assert torch.equal(h, r)
        else:
            assert relerr(h.numpy(), r.numpy()) < 1e-10
    assert a.itime == b.itime == 6
