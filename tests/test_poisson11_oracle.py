"""poisson_11x (src/poisson.f90:1019-1465): free-slip x and y, z free-slip or
periodic, in the oracle.

* the solve inverts the discrete div(grad) of the free-slip staggered
  operators (divergence / gradp with ncl = 1) to round-off, for both z cases;
* the reference's golden vector itself, tests/TGV-Taylor-Green-vortex/
  reference_time_evol.dat (65^3 free-slip box [0, pi]^3, RK3, dt = 0.005),
  run directly on the free-slip box: the first 5 rows (50 steps) within
  1e-10 relative (the file prints 12 digits)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD64 = np.loadtxt(os.path.join(HERE, "golden", "tgv_freeslip65_rk3_fp64.txt"))


@pytest.mark.parametrize("bcz", [1, 0])
def test_poisson_11x_inverts_div_grad(oracle_mod, bcz):
    n, L = 33, np.pi
    nz = 33 if bcz else 32
    o = oracle_mod.Oracle(n, n, nz, L, L, L, bc=((1, 1), (1, 1), (bcz, bcz)))
    p = np.random.default_rng(5).standard_normal((nz - bcz, n - 1, n - 1))
    rhs = o.divergence(*o.gradp(p))
    q = o.poisson(rhs.copy())
    d = (q - q.mean()) - (p - p.mean())
    assert np.abs(d).max() < 1e-13 * np.abs(p).max()


def freeslip_tgv(n):
    x = np.arange(n) * (np.pi / (n - 1))
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    return np.sin(X) * np.cos(Y) * np.cos(Z), -np.cos(X) * np.sin(Y) * np.cos(Z), np.zeros((n, n, n))


def test_oracle_reproduces_reference_directly_on_the_freeslip_box(oracle_mod):
    n, L = 65, np.pi
    o = oracle_mod.Oracle(n, n, n, L, L, L, bc=((1, 1), (1, 1), (1, 1)))
    _, _, _, rows, divmax = o.run(*freeslip_tgv(n), 50, 0.005, 1.0 / 1600.0, 5, 10)
    assert np.allclose(rows[:, 0], GOLD64[:5, 0])
    rel = np.abs(rows[:, 1:] - GOLD64[:5, 1:]) / np.abs(GOLD64[:5, 1:])
    assert np.all(rel < 1e-10), rel
    assert divmax < 1e-11


def test_freeslip_bench_cpu_leg_times_the_oracle_on_the_same_case(oracle_mod):
    """bench.py --workload freeslip reports the oracle on the same free-slip
    box beside the GPU rate (here on a small grid, one step)."""
    import bench
    out = bench.freeslip_cpu_baseline(np, 17, np.pi, 0.005, steps=1)
    assert out["kind"] == "port" and out["cores"] >= 1 and out["value"] > 0
    assert "17^3 free-slip" in out["sample"]
