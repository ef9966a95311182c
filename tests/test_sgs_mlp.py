"""Learned SGS closure: the MLP kernels against a numpy statement of the same
network, the ratio-4 box filter against numpy, and the solver's SGS force
against the library's own operators (GPU)."""
import math

import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu
L = 2 * np.pi


def erf(x):
    return np.vectorize(math.erf)(x)


def np_forward(P, sc, X):
    """(pre-activations, activations, outputs) of the 10-64-64-6 GELU network."""
    W1 = P[:640].reshape(64, 10)
    b1 = P[640:704]
    W2 = P[704:4800].reshape(64, 64)
    b2 = P[4800:4864]
    W3 = P[4864:5248].reshape(6, 64)
    b3 = P[5248:5254]
    x = X * sc[:10]
    a1 = x @ W1.T + b1
    h1 = 0.5 * a1 * (1 + erf(a1 / math.sqrt(2)))
    a2 = h1 @ W2.T + b2
    h2 = 0.5 * a2 * (1 + erf(a2 / math.sqrt(2)))
    y = h2 @ W3.T + b3
    return x, a1, h1, a2, h2, y


def np_grad(P, sc, X, T, lam=0.0, pscale=1.0):
    x, a1, h1, a2, h2, y = np_forward(P, sc, X)
    n = X.shape[0]
    W2 = P[704:4800].reshape(64, 64)
    W3 = P[4864:5248].reshape(6, 64)
    gd = lambda a: 0.5 * (1 + erf(a / math.sqrt(2))) + a * np.exp(-0.5 * a * a) / math.sqrt(2 * math.pi)  # noqa
    dy = 2 * (y - T / sc[10:]) / n
    if lam:
        # energy flux Pi = tau_ij S_ij with S from the raw gradient features
        S = np.stack([X[:, 0], X[:, 4], X[:, 8], 0.5 * (X[:, 1] + X[:, 3]), 0.5 * (X[:, 2] + X[:, 6]),
                      0.5 * (X[:, 5] + X[:, 7])], axis=1)
        w = np.array([1, 1, 1, 2, 2, 2.0])
        e = ((y * sc[10:] * w * S).sum(1) - (T * w * S).sum(1)) / pscale
        dy = dy + 2 * lam * e[:, None] * w * S * sc[10:] / pscale / n
    d2 = (dy @ W3) * gd(a2)
    d1 = (d2 @ W2) * gd(a1)
    return np.concatenate([(d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), (dy.T @ h2).ravel(),
                           dy.sum(0)])


@pytest.fixture
def mlp(gpu_lib):
    from incompact3d_gb300 import sgs
    m = sgs.Mlp(seed=3)
    rng = np.random.default_rng(4)
    sc = np.concatenate([rng.uniform(0.5, 2, 10), rng.uniform(0.5, 2, 6)]).astype(np.float32)
    m.set(sgs.init_params(3), sc)
    yield m
    m.close()


def test_inference_matches_numpy(mlp):
    import torch
    P, sc = mlp.get()
    X = np.random.default_rng(5).standard_normal((1000, 10)).astype(np.float32)
    Y = mlp.infer(torch.from_numpy(X).cuda()).cpu().numpy()
    ref = np_forward(P.astype(np.float64), sc.astype(np.float64), X.astype(np.float64))[-1] * sc[10:]
    assert np.abs(Y - ref).max() < 2e-5 * np.abs(ref).max()


def test_first_adam_step_follows_gradient_sign(mlp):
    # Adam's first step moves every parameter by -lr * g / (|g| + eps): the
    # sign of the kernel's batch gradient equals numpy's wherever |g| is clear
    import torch
    P0, sc = mlp.get()
    rng = np.random.default_rng(6)
    X = rng.standard_normal((3000, 10)).astype(np.float32)
    T = rng.standard_normal((3000, 6)).astype(np.float32)
    mlp.train_step(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda(), 1e-3)
    P1, _ = mlp.get()
    g = np_grad(P0.astype(np.float64), sc.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    big = np.abs(g) > 1e-4 * np.abs(g).max()
    step = P1 - P0
    assert np.all(np.sign(step[big]) == -np.sign(g[big]))
    np.testing.assert_allclose(np.abs(step[big]), 1e-3, rtol=1e-2)


def test_first_adam_step_with_flux_loss(mlp):
    import torch
    P0, sc = mlp.get()
    rng = np.random.default_rng(9)
    X = rng.standard_normal((3000, 10)).astype(np.float32)
    T = rng.standard_normal((3000, 6)).astype(np.float32)
    mlp.set_flux_loss(2.0, 3.0)
    mlp.train_step(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda(), 1e-3)
    P1, _ = mlp.get()
    g = np_grad(P0.astype(np.float64), sc.astype(np.float64), X.astype(np.float64), T.astype(np.float64), 2.0, 3.0)
    g0 = np_grad(P0.astype(np.float64), sc.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    big = np.abs(g) > 1e-4 * np.abs(g).max()
    step = P1 - P0
    assert np.all(np.sign(step[big]) == -np.sign(g[big]))
    # the flux term changes the direction of a share of the parameters
    assert np.mean(np.sign(g[big]) != np.sign(g0[big])) > 0.05


def test_flux_loss_rejects_bad_arguments(mlp):
    with pytest.raises(Exception):
        mlp.set_flux_loss(1.0, 0.0)
    with pytest.raises(Exception):
        mlp.set_flux_loss(-1.0, 1.0)


def test_training_fits_a_smooth_map(mlp):
    import torch
    rng = np.random.default_rng(7)
    X = rng.standard_normal((65536, 10)).astype(np.float32)
    A = rng.standard_normal((10, 6)).astype(np.float32) * 0.3
    T = np.tanh(X @ A).astype(np.float32)
    mlp.set(None, np.ones(16, np.float32))
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    first = mlp.train_step(Xd[:8192], Td[:8192], 3e-3, want_loss=True)
    for it in range(400):
        i0 = (it % 8) * 8192
        mlp.train_step(Xd[i0:i0 + 8192], Td[i0:i0 + 8192], 3e-3)
    last = mlp.train_step(Xd[:8192], Td[:8192], 1e-4, want_loss=True)
    assert last < 0.05 * first


def np_box4(u):
    w = np.array([0.5, 1, 1, 1, 0.5]) / 4
    n = u.shape[0]
    out = np.zeros((n // 4,) * 3)
    for a in range(5):
        for b in range(5):
            for c in range(5):
                sh = np.roll(u, (2 - c, 2 - b, 2 - a), axis=(0, 1, 2))
                out += w[a] * w[b] * w[c] * sh[::4, ::4, ::4]
    return out


def test_box_filter_matches_numpy(gpu_lib):
    import torch
    from incompact3d_gb300 import _lib, sgs
    rng = np.random.default_rng(8)
    u = [rng.standard_normal((16, 16, 16)) for _ in range(3)]
    ub, tau = sgs.box_filter4(_lib.load(), *[torch.from_numpy(a).cuda() for a in u])
    for q in range(3):
        assert relerr(ub[q].cpu().numpy(), np_box4(u[q])) < 1e-14
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    for q, (i, j) in enumerate(pairs):
        ref = np_box4(u[i] * u[j]) - np_box4(u[i]) * np_box4(u[j])
        assert relerr(tau[q].cpu().numpy(), ref) < 1e-13


def test_solver_sgs_force_is_divergence_of_mlp_stress(gpu_lib, mlp):
    import torch
    from incompact3d_gb300 import _lib, sgs
    from test_les import tgv
    n = 32
    c = gpu_lib.Context(n, n, n, L, L, L)
    s = gpu_lib.Solver(c, 0.005, 1 / 5000.0, itimescheme=3, precision=gpu_lib.PREC_FP64)
    u = tgv(n, noise=0.05)
    s.set_velocity(*u)
    _lib.check(_lib.load().x3d_solver_set_les_mlp(s.h, mlp.h))
    nut, fx, fy, fz = [t.cpu().numpy() for t in s.les_fields()]
    ud = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in u]
    X, delta = sgs.features(c, ud)
    tau = mlp.infer(X).double().t().reshape(6, n, n, n)
    ti = [[0, 3, 4], [3, 1, 5], [4, 5, 2]]
    pt = [[1, 1, 1], [1, 1, 1], [1, 1, 1], [0, 0, 1], [0, 1, 0], [1, 0, 0]]
    for i, f in enumerate((fx, fy, fz)):
        ref = -sum(c.apply(j, gpu_lib.OP_DER1, pt[ti[i][j]][j], tau[ti[i][j]].contiguous()).cpu().numpy()
                   for j in range(3))
        assert relerr(f, ref) < 1e-12
    assert np.all(nut == 0)
