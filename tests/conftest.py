import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libx3dgpu.so kernels)")
    config.addinivalue_line("markers", "slow: long-running CPU oracle case")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib_host():
    """Built library for host-side calls (context tables); no device needed."""
    import incompact3d_gb300 as x3d
    x3d.build()
    x3d.load()
    return x3d


@pytest.fixture(scope="session")
def gpu_lib():
    """Built library + a CUDA device; the library is the only compute path."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import incompact3d_gb300 as x3d
    x3d.build()
    x3d.load()
    return x3d


def grid_coords(n, L, periodic):
    d = L / n if periodic else L / (n - 1)
    return np.arange(n) * d


def fourier_field(nx, ny, nz, L=(2 * np.pi,) * 3, nmodes=12, kmax=4, seed=1, periodic=(True,) * 3):
    """Smooth seeded field: sum of random Fourier modes, shape (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    x = grid_coords(nx, L[0], periodic[0])[None, None, :]
    y = grid_coords(ny, L[1], periodic[1])[None, :, None]
    z = grid_coords(nz, L[2], periodic[2])[:, None, None]
    f = np.zeros((nz, ny, nx))
    for _ in range(nmodes):
        k = rng.integers(-kmax, kmax + 1, size=3)
        ph = rng.uniform(0, 2 * np.pi)
        a = rng.uniform(0.2, 1.0)
        f += a * np.cos(k[0] * x * 2 * np.pi / L[0] + k[1] * y * 2 * np.pi / L[1] + k[2] * z * 2 * np.pi / L[2] + ph)
    return f


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
