"""Channel path on the GPU vs the oracle: stretched-mesh y operators,
poisson_010 (uniform and stretched y, src/poisson.f90:665-1013 with
matrice_refinement and inversion5_v1), the projection pieces, and the
channel time loop (constant flow rate, no-slip walls, RK3).

Tolerances: operators and Poisson 1e-12 relative (FP64); velocity after the
time loop 1e-10 relative.  The full-size workload 256x129x128 (Lx = 8 pi,
Ly = 2, Lz = 3 pi, istret = 2, beta = 0.259) is checked through
size-independent properties: the projection leaves max|div u| at round-off and
the flow-rate control holds the bulk velocity at 2/3.
"""
import ctypes

import numpy as np
import pytest

from conftest import relerr
from test_channel_oracle import BETA, channel_ic, smooth_pressure

pytestmark = pytest.mark.gpu
CH = ((0, 0), (2, 2), (0, 0))


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def pair(oracle_mod, gpu_lib, n, L, istret):
    o = oracle_mod.Oracle(*n, *L, bc=CH, istret=istret, beta=BETA)
    c = gpu_lib.Context(*n, *L, bc=CH, istret=istret, beta=BETA)
    return o, c


@pytest.mark.parametrize("istret", [0, 2])
@pytest.mark.parametrize("npaire", [0, 1])
def test_dery_stretched(oracle_mod, gpu_lib, istret, npaire):
    import torch
    n, L = (32, 33, 16), (4.0, 2.0, 3.0)
    o, c = pair(oracle_mod, gpu_lib, n, L, istret)
    rng = np.random.default_rng(5)
    u = rng.standard_normal((n[2], n[1], n[0]))
    ppy = c.stretching()["ppy"]
    ref = o.op(1, oracle_mod.OP_DER1, npaire, u, pp=ppy if istret else None)
    t = torch.empty((n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    fs = "P" if npaire == 1 else ""
    c.dery(t, dev(torch, u), ffy=c.coeffs(1, "FF" + fs), fsy=c.coeffs(1, "FS" + fs), fwy=c.coeffs(1, "FW" + fs),
           ppy=ppy, npaire=npaire)
    assert relerr(t.cpu().numpy(), ref) < 1e-12


def test_dery_rejects_foreign_ppy(gpu_lib):
    import torch
    c = gpu_lib.Context(16, 17, 8, 4.0, 2.0, 3.0, bc=CH, istret=2, beta=BETA)
    u = torch.zeros((8, 17, 16), dtype=torch.float64, device="cuda")
    with pytest.raises(gpu_lib.X3DError):
        c.dery(torch.empty_like(u), u, ppy=np.ones(17))


@pytest.mark.parametrize("istret", [0, 2])
def test_divergence_gradp_stretched(oracle_mod, gpu_lib, istret):
    import torch
    n, L = (32, 33, 16), (4.0, 2.0, 3.0)
    o, c = pair(oracle_mod, gpu_lib, n, L, istret)
    rng = np.random.default_rng(6)
    ux, uy, uz = [rng.standard_normal((n[2], n[1], n[0])) for _ in range(3)]
    d_ref = o.divergence(ux, uy, uz)
    d = c.divergence(dev(torch, ux), dev(torch, uy), dev(torch, uz))
    assert relerr(d.cpu().numpy(), d_ref) < 1e-12
    p = rng.standard_normal(d_ref.shape)
    g_ref = o.gradp(p)
    g = c.gradp(dev(torch, p))
    for a, b in zip(g, g_ref):
        assert relerr(a.cpu().numpy(), b) < 1e-12


@pytest.mark.parametrize("istret", [0, 1, 2])
@pytest.mark.parametrize("n", [(32, 33, 16), (64, 65, 32), (16, 129, 8)])
def test_poisson010_matches_oracle(oracle_mod, gpu_lib, istret, n):
    import torch
    L = (4.0, 2.0, 3.0)
    o, c = pair(oracle_mod, gpu_lib, n, L, istret)
    rng = np.random.default_rng(7)
    r = rng.standard_normal((n[2], n[1] - 1, n[0]))
    ref = o.poisson(r)
    x = dev(torch, r)
    c.poisson(x)
    assert relerr(x.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("istret", [0, 2])
def test_poisson010_full_size_inverts_div_grad(gpu_lib, istret):
    import torch
    n, L = (256, 129, 128), (8 * np.pi, 2.0, 3 * np.pi)
    c = gpu_lib.Context(*n, *L, bc=CH, istret=istret, beta=BETA)
    p0 = smooth_pressure(n[0], n[1] - 1, n[2], L, nmodes=8)
    g = c.gradp(dev(torch, p0))
    r = c.divergence(*g)
    c.poisson(r)
    p1 = r.cpu().numpy()
    err = np.abs((p1 - p1.mean()) - (p0 - p0.mean())).max()
    assert err < 1e-11 * np.abs(p0).max(), err


def run_pair(oracle_mod, gpu_lib, n, L, istret, nsteps, itimescheme=5, wrot=0.0, spin=0):
    o, c = pair(oracle_mod, gpu_lib, n, L, istret)
    ic = channel_ic(n[0], n[1], n[2], L[1], c.stretching()["yp"])
    ref = o.run_channel(*ic, nsteps, 0.002, 1 / 4200.0, itimescheme=itimescheme, wrotation=wrot,
                        spinup_time=spin)
    s = gpu_lib.Solver(c, 0.002, 1 / 4200.0, itimescheme=itimescheme, precision=gpu_lib.PREC_FP64)
    s.set_channel(2.0 / 3.0, wrot, spin)
    s.set_velocity(*ic)
    ub = []
    for _ in range(nsteps):
        s.step(1)
        ub.extend(s.bulk_velocity())
    return ref, s.get_velocity(), np.array(ub), s


@pytest.mark.parametrize("istret", [0, 2])
def test_channel_rk3_matches_oracle(oracle_mod, gpu_lib, istret):
    n, L = (32, 33, 16), (2 * np.pi, 2.0, np.pi)
    ref, u, ub, s = run_pair(oracle_mod, gpu_lib, n, L, istret, 10)
    for a, b in zip(u, ref[:3]):
        assert relerr(a, b) < 1e-10
    np.testing.assert_allclose(ub, ref[3], rtol=1e-12, atol=0)
    assert s.divmax() < 1e-11


def test_channel_ab3_rotation_matches_oracle(oracle_mod, gpu_lib):
    n, L = (32, 33, 16), (2 * np.pi, 2.0, np.pi)
    ref, u, ub, s = run_pair(oracle_mod, gpu_lib, n, L, 2, 8, itimescheme=3, wrot=0.12, spin=5)
    for a, b in zip(u, ref[:3]):
        assert relerr(a, b) < 1e-10
    np.testing.assert_allclose(ub, ref[3], rtol=1e-12, atol=0)


def test_channel_full_size_properties(gpu_lib):
    n, L = (256, 129, 128), (8 * np.pi, 2.0, 3 * np.pi)
    c = gpu_lib.Context(*n, *L, bc=CH, istret=2, beta=BETA)
    s = gpu_lib.Solver(c, 0.002, 1 / 4200.0, itimescheme=5, precision=gpu_lib.PREC_FP64)
    s.set_channel()
    s.set_velocity(*channel_ic(n[0], n[1], n[2], L[1], c.stretching()["yp"]))
    s.step(5)
    ub = s.bulk_velocity()
    assert np.all(np.abs(ub - 2.0 / 3.0) < 1e-3)
    assert s.divmax() < 1e-10
    u = s.get_velocity()
    assert np.all(u[1][:, 0, :] == 0) and np.all(u[1][:, -1, :] == 0)
    assert np.all(np.isfinite(u[0]))
