"""Pin against the reference's only golden vector.

The reference's TGV regression test (tests/TGV-Taylor-Green-vortex: 65^3
free-slip box [0, pi]^3, Re=1600, RK3, dt=0.005, 500 steps; fixtures in
tests/golden/, made by make_tgv_golden.py) is the mirror-symmetric half of the
triply periodic 128^3 TGV on [0, 2 pi]^3 at the same grid spacing: the
free-slip closures of the compact schemes, the mirrored staggered operators
and the cosine-transform Poisson solve of poisson_11x are the periodic
operators applied to the symmetric extension, and the reference averages its
statistics over the 64^3 points of the half box, which equal the 128^3
periodic averages for the TGV symmetries.  So the periodic path reproduces the
reference's own output:

* CPU oracle, first row (10 steps), within 1e-10 (the file prints 12 digits);
* GPU FP64 solver through the C ABI, all 50 rows, within rtol 1e-7 - the
  tolerance of the reference's own comparator
  (tests/TGV-Taylor-Green-vortex/compare_TGV_time_evolution.py) - and in
  practice ~1e-11;
* GPU mixed-precision solver: kinetic energy within 1e-6 of the FP64 file.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD64 = np.loadtxt(os.path.join(HERE, "golden", "tgv_freeslip65_rk3_fp64.txt"))
GOLD32 = np.loadtxt(os.path.join(HERE, "golden", "tgv_freeslip65_rk3_fp32.txt"))
L = 2 * np.pi
N = 128
DT = 0.005
XNU = 1.0 / 1600.0


def tgv_ic(n):
    x = np.arange(n) * (L / n)
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    return np.sin(X) * np.cos(Y) * np.cos(Z), -np.cos(X) * np.sin(Y) * np.cos(Z), np.zeros((n, n, n))


def test_golden_vectors_are_consistent():
    assert GOLD64.shape == (50, 5) and GOLD32.shape == (50, 5)
    assert np.allclose(GOLD64[:, 0], (np.arange(1, 51) * 10 - 1) * DT)
    # the FP32 build of the reference agrees with the FP64 build to its 6 printed digits
    assert np.max(np.abs(GOLD32[:, 1] - GOLD64[:, 1])) < 1e-6


def test_oracle_reproduces_reference_first_row(oracle_mod):
    o = oracle_mod.Oracle(N, N, N, L, L, L)
    _, _, _, rows, _ = o.run(*tgv_ic(N), 10, DT, XNU, 5, 10)
    rel = np.abs(rows[0, 1:] - GOLD64[0, 1:]) / np.abs(GOLD64[0, 1:])
    assert rows[0, 0] == pytest.approx(GOLD64[0, 0])
    assert np.all(rel < 1e-10), rel


@pytest.mark.gpu
def test_gpu_fp64_reproduces_reference_time_evolution(gpu_lib):
    ctx = gpu_lib.Context(N, N, N, L, L, L)
    s = gpu_lib.Solver(ctx, DT, XNU, itimescheme=5, precision=gpu_lib.PREC_FP64)
    s.set_velocity(*tgv_ic(N))
    rows = []
    for it in range(1, 501):
        s.step(1)
        if it % 10 == 0:
            rows.append([(it - 1) * DT, *s.tgv_stats()])
    rows = np.array(rows)
    np.testing.assert_allclose(rows, GOLD64, rtol=1e-7, atol=0)
    assert np.max(np.abs(rows[:, 1:] - GOLD64[:, 1:]) / np.abs(GOLD64[:, 1:])) < 1e-9
    assert s.divmax() < 1e-11


@pytest.mark.gpu
def test_gpu_mixed_precision_energy_vs_reference(gpu_lib):
    ctx = gpu_lib.Context(N, N, N, L, L, L)
    s = gpu_lib.Solver(ctx, DT, XNU, itimescheme=5, precision=gpu_lib.PREC_MIXED)
    s.set_velocity(*tgv_ic(N))
    ek = []
    for it in range(1, 501):
        s.step(1)
        if it % 10 == 0:
            ek.append(s.tgv_stats()[0])
    assert np.max(np.abs(np.array(ek) - GOLD64[:, 1])) < 1e-6
