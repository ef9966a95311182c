"""Tensor-core (tcgen05) inference of the learned SGS closure.

The three layers run as M = 128 MMAs on BF16 hi / lo split operands
(hi*hi + hi*lo + lo*hi, FP32 accumulation in tensor memory).  Against the
network evaluated in binary64 (numpy) every output is within 1e-4 of the
largest output magnitude, and within the same bound of the FP32 CUDA-core
kernel; ragged point counts (not multiples of the 128-point tile) and the
repacking of the weights after a training step are covered, as is the
solver's closure force with the tensor-core path selected."""
import numpy as np
import pytest

from conftest import relerr
from test_sgs_mlp import np_forward

pytestmark = pytest.mark.gpu
L = 2 * np.pi
TOL = 1e-4


def make_mlp(seed):
    from incompact3d_gb300 import sgs
    m = sgs.Mlp(seed=seed)
    rng = np.random.default_rng(seed + 1)
    P = sgs.init_params(seed)
    P[640:704] = rng.uniform(-0.5, 0.5, 64)      # b1
    P[4800:4864] = rng.uniform(-0.5, 0.5, 64)    # b2
    P[5248:5254] = rng.uniform(-0.5, 0.5, 6)     # b3
    sc = np.concatenate([rng.uniform(0.5, 2, 10), rng.uniform(0.5, 2, 6)]).astype(np.float32)
    m.set(P, sc)
    return m


def infer_both(m, X):
    m.set_tensor_cores(False)
    y32 = m.infer(X).cpu().numpy()
    m.set_tensor_cores(True)
    ytc = m.infer(X).cpu().numpy()
    m.status()
    return y32, ytc


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 70001])
def test_tensor_core_inference_matches_binary64_network(gpu_lib, n):
    import torch
    m = make_mlp(7)
    X = np.random.default_rng(n).standard_normal((n, 10)).astype(np.float32)
    y32, ytc = infer_both(m, torch.from_numpy(X).cuda())
    P, sc = m.get()
    ref = np_forward(P.astype(np.float64), sc.astype(np.float64), X.astype(np.float64))[-1] * sc[10:]
    scale = np.abs(ref).max()
    assert np.abs(ytc - ref).max() < TOL * scale
    assert np.abs(ytc - y32).max() < TOL * scale
    m.close()


def test_tensor_core_weights_follow_training_steps(gpu_lib):
    import torch
    m = make_mlp(11)
    rng = np.random.default_rng(12)
    X = torch.from_numpy(rng.standard_normal((4096, 10)).astype(np.float32)).cuda()
    T = torch.from_numpy(rng.standard_normal((4096, 6)).astype(np.float32)).cuda()
    m.set_tensor_cores(True)
    before = m.infer(X).cpu().numpy()
    for _ in range(3):
        m.train_step(X, T, 1e-2)
    y32, ytc = infer_both(m, X)
    assert np.abs(ytc - y32).max() < TOL * np.abs(y32).max()
    assert np.abs(ytc - before).max() > 100 * TOL * np.abs(y32).max()  # the new weights were used
    m.close()


def test_solver_closure_on_tensor_cores_matches_fp32(gpu_lib):
    from incompact3d_gb300 import _lib
    from test_les import tgv
    n = 32
    c = gpu_lib.Context(n, n, n, L, L, L)
    u = tgv(n, noise=0.05)
    m = make_mlp(5)
    forces = []
    for on in (False, True):
        m.set_tensor_cores(on)
        s = gpu_lib.Solver(c, 0.005, 1 / 5000.0, itimescheme=3, precision=gpu_lib.PREC_FP64)
        s.set_velocity(*u)
        _lib.check(_lib.load().x3d_solver_set_les_mlp(s.h, m.h))
        forces.append([t.cpu().numpy() for t in s.les_fields()[1:]])
        s.close()
    m.status()
    for a, b in zip(*forces):
        assert relerr(b, a) < 10 * TOL
    m.close()
