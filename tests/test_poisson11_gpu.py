"""poisson_11x on the GPU (src/poisson.f90:1019-1465): free-slip x and y, z
free-slip or periodic, FP64.

* against the oracle on the same right-hand side: 1e-12 of the largest value;
* inverts the discrete div(grad) of the GPU's own free-slip staggered
  operators to round-off;
* the free-slip TGV (the reference's regression case: 65^3 box [0, pi]^3,
  Re = 1600, RK3, dt = 0.005, 500 steps) run directly through the solver:
  all 50 rows of tests/TGV-Taylor-Green-vortex/reference_time_evol.dat within
  rtol 1e-7, the tolerance of the reference's own comparator."""
import os

import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD64 = np.loadtxt(os.path.join(HERE, "golden", "tgv_freeslip65_rk3_fp64.txt"))


def cases():
    return [((33, 33, 33), 1), ((65, 33, 17), 1), ((33, 65, 32), 0), ((129, 65, 33), 1)]


@pytest.mark.parametrize("dims,bcz", cases())
def test_poisson_11x_matches_oracle(gpu_lib, oracle_mod, dims, bcz):
    import torch
    nx, ny, nz = dims
    L = np.pi
    bc = ((1, 1), (1, 1), (bcz, bcz))
    ctx = gpu_lib.Context(nx, ny, nz, L, 2.0, 1.5, bc=bc)
    o = oracle_mod.Oracle(nx, ny, nz, L, 2.0, 1.5, bc=bc)
    shp = (nz - bcz, ny - 1, nx - 1)
    rhs = np.random.default_rng(nx + ny + nz).standard_normal(shp)
    ref = o.poisson(rhs.copy())
    got = ctx.poisson(torch.from_numpy(rhs).cuda()).cpu().numpy()
    assert relerr(got, ref) < 1e-12


@pytest.mark.parametrize("bcz", [1, 0])
def test_poisson_11x_inverts_gpu_div_grad(gpu_lib, bcz):
    import torch
    n = 65
    nz = n if bcz else 64
    ctx = gpu_lib.Context(n, n, nz, np.pi, np.pi, np.pi, bc=((1, 1), (1, 1), (bcz, bcz)))
    p = torch.from_numpy(np.random.default_rng(3).standard_normal((nz - bcz, n - 1, n - 1))).cuda()
    rhs = ctx.divergence(*ctx.gradp(p))
    q = ctx.poisson(rhs.clone())
    d = (q - q.mean()) - (p - p.mean())
    assert float(d.abs().max()) < 1e-12 * float(p.abs().max())


def freeslip_tgv(n):
    x = np.arange(n) * (np.pi / (n - 1))
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    return np.sin(X) * np.cos(Y) * np.cos(Z), -np.cos(X) * np.sin(Y) * np.cos(Z), np.zeros((n, n, n))


def test_gpu_reproduces_reference_time_evolution_on_the_freeslip_box(gpu_lib):
    n, L = 65, np.pi
    ctx = gpu_lib.Context(n, n, n, L, L, L, bc=((1, 1), (1, 1), (1, 1)))
    s = gpu_lib.Solver(ctx, 0.005, 1.0 / 1600.0, itimescheme=5, precision=gpu_lib.PREC_FP64)
    s.set_velocity(*freeslip_tgv(n))
    rows = []
    for it in range(1, 501):
        s.step(1)
        if it % 10 == 0:
            rows.append([(it - 1) * 0.005, *s.tgv_stats()])
    rows = np.array(rows)
    np.testing.assert_allclose(rows, GOLD64, rtol=1e-7, atol=0)
    assert np.max(np.abs(rows[:, 1:] - GOLD64[:, 1:]) / np.abs(GOLD64[:, 1:])) < 1e-9
    assert s.divmax() < 1e-11


def test_mixed_precision_is_refused_on_the_freeslip_box(gpu_lib):
    from incompact3d_gb300._lib import X3DError
    ctx = gpu_lib.Context(33, 33, 33, np.pi, np.pi, np.pi, bc=((1, 1), (1, 1), (1, 1)))
    with pytest.raises(X3DError):
        gpu_lib.Solver(ctx, 0.005, 1.0 / 1600.0, itimescheme=5, precision=gpu_lib.PREC_MIXED)
