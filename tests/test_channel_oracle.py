"""Oracle checks for the channel path (CPU): stretched-mesh metrics
(src/stretching.f90), poisson_010 with and without the pentadiagonal
stretched-mesh solve (src/poisson.f90:665-1013, 1814-2113, src/tools.f90:
1225-1362) and the constant-flow-rate channel time loop.

poisson_010 is pinned by exactness: for resolved pressure modes the solve must
invert the discrete divergence-of-gradient of the staggered compact operators
(the reference's machine-precision divergence claim), on uniform and
stretched meshes.
"""
import numpy as np
import pytest

BETA = 0.259065151


def smooth_pressure(nx, nym, nz, L, seed=1, nmodes=6):
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * L[0] / nx
    y = (np.arange(nym) + 0.5) * L[1] / nym
    z = np.arange(nz) * L[2] / nz
    p = np.zeros((nz, nym, nx))
    for _ in range(nmodes):
        kx, m, kz = rng.integers(0, 4), rng.integers(0, 5), rng.integers(0, 3)
        ph = rng.uniform(0, 2 * np.pi, 2)
        p += (np.cos(2 * np.pi * kx * x / L[0] + ph[0])[None, None, :] * np.cos(np.pi * m * y / L[1])[None, :, None]
              * np.cos(2 * np.pi * kz * z / L[2] + ph[1])[:, None, None])
    return p


def channel_ic(nx, ny, nz, Ly, yp, noise=0.125, seed=20261204):
    """Laminar Poiseuille profile plus modulated uniform noise
    (src/Case-Channel.f90:104-130 with a seeded PCG64 stream)."""
    rng = np.random.default_rng(seed)
    y = yp - Ly / 2
    um = np.exp(-0.2 * y * y)
    r = [rng.uniform(size=(nz, ny, nx)) for _ in range(3)]
    ux = noise * um[None, :, None] * (2 * r[0] - 1) + (1 - y * y)[None, :, None]
    uy = noise * um[None, :, None] * (2 * r[1] - 1)
    uz = noise * um[None, :, None] * (2 * r[2] - 1)
    return ux, uy, uz


@pytest.mark.parametrize("istret", [1, 2, 3])
def test_stretching_metrics(oracle_mod, istret):
    ny = 129
    o = oracle_mod.Oracle(8, ny, 8, 4.0, 2.0, 3.0, bc=((0, 0), (2, 2), (0, 0)), istret=istret, beta=BETA)
    st = o.stretching()
    yp = st["yp"]
    assert yp[0] == 0.0
    assert np.all(np.diff(yp) > 0)
    top = 2.0 if istret != 3 else 2.0 * 2.0 / 2.0
    assert abs(yp[-1] - top) < 1e-12
    np.testing.assert_allclose(st["pp2y"], st["ppy"] ** 2, rtol=0, atol=0)
    if istret == 2:
        # refined at both walls: symmetric about the centre line
        np.testing.assert_allclose(yp + yp[::-1], 2.0, atol=1e-12)
    # ppy is Ly * deta/dy: finite differences of the mapping agree with it
    deta = 1.0 / (ny - 1) if istret != 3 else 0.5 / (ny - 1)
    dyde = np.gradient(yp, deta * (1 if istret != 3 else 2))
    mid = slice(4, -4)
    np.testing.assert_allclose((dyde * st["ppy"] / 2.0)[mid], 1.0, rtol=2e-3)


def test_uniform_ppy_defaults(oracle_mod):
    o = oracle_mod.Oracle(8, 9, 8, 4.0, 2.0, 3.0, bc=((0, 0), (2, 2), (0, 0)))
    st = o.stretching()
    assert st["ppy"][0] == 2.0 and st["ppy"][-1] == 2.0 and np.all(st["ppy"][1:-1] == 1.0)


@pytest.mark.parametrize("istret", [0, 1, 2])
def test_poisson010_inverts_div_grad(oracle_mod, istret):
    nx, ny, nz = 16, 17, 8
    L = (4.0, 2.0, 3.0)
    o = oracle_mod.Oracle(nx, ny, nz, *L, bc=((0, 0), (2, 2), (0, 0)), istret=istret, beta=BETA)
    p0 = smooth_pressure(nx, ny - 1, nz, L)
    r = o.divergence(*o.gradp(p0))
    p1 = o.poisson(r)
    err = np.abs((p1 - p1.mean()) - (p0 - p0.mean())).max()
    assert err < 1e-12 * np.abs(p0).max(), err


@pytest.mark.parametrize("istret", [0, 2])
def test_channel_projection_and_flow_rate(oracle_mod, istret):
    nx, ny, nz = 16, 17, 8
    o = oracle_mod.Oracle(nx, ny, nz, 2 * np.pi, 2.0, np.pi, bc=((0, 0), (2, 2), (0, 0)), istret=istret, beta=BETA)
    ux, uy, uz = channel_ic(nx, ny, nz, 2.0, o.stretching()["yp"])
    a, b, c, ub, dmax = o.run_channel(ux, uy, uz, 4, 0.002, 1 / 4200.0, itimescheme=5)
    assert len(ub) == 12
    assert abs(ub[-1] - 2.0 / 3.0) < 1e-5
    assert dmax < 1e-12
    assert np.all(b[:, 0, :] == 0) and np.all(b[:, -1, :] == 0)


@pytest.mark.parametrize("istret", [0, 1, 2, 3])
def test_library_stretching_tables_match_oracle(oracle_mod, gpu_lib_host, istret):
    """The library's host-side stretching metrics equal the oracle's bit for bit
    (no device needed: the context builds its tables on the host)."""
    ny = 65
    L = (8 * np.pi, 2.0, 3 * np.pi)
    o = oracle_mod.Oracle(32, ny, 16, *L, bc=((0, 0), (2, 2), (0, 0)), istret=istret, beta=BETA)
    ctx = gpu_lib_host.Context(32, ny, 16, *L, bc=((0, 0), (2, 2), (0, 0)), istret=istret, beta=BETA)
    a, b = o.stretching(), ctx.stretching()
    for k in ("yp", "ypi", "ppy", "pp2y", "pp4y", "ppyi", "pp2yi", "pp4yi"):
        assert np.array_equal(a[k], b[k]), k
    assert a["alpha"] == b["alpha"]
