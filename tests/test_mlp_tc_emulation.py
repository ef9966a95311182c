"""CPU replay of the tensor-core inference arithmetic of the SGS closure: every
operand x carried as bf16(x) + bf16(x - bf16(x)), products hi*hi + hi*lo +
lo*hi summed in binary32.  The replay stays within 1e-4 of the largest
output of the binary64 network, the bound the GPU test asserts."""
import math

import numpy as np

from test_sgs_mlp import np_forward


def bf16(x):
    """Round binary32 to bfloat16 (nearest, ties to even), returned as binary32."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def split(x):
    x = np.asarray(x, dtype=np.float32)
    h = bf16(x)
    return h, bf16(x - h)


def mm3(A, W):
    """A (m, k) times W (n, k)^T from split parts, binary32 accumulation."""
    ah, al = split(A)
    wh, wl = split(W)
    f = np.float32
    return (ah.astype(f) @ wh.T.astype(f) + ah @ wl.T + al @ wh.T).astype(f)


def gelu32(a):
    erf = np.vectorize(math.erf)
    return (0.5 * a * (1 + erf(a / math.sqrt(2)))).astype(np.float32)


def tc_forward(P, sc, X):
    W1 = P[:640].reshape(64, 10)
    b1 = P[640:704]
    W2 = P[704:4800].reshape(64, 64)
    b2 = P[4800:4864]
    W3 = P[4864:5248].reshape(6, 64)
    b3 = P[5248:5254]
    x = (X * sc[:10]).astype(np.float32)
    h1 = gelu32(mm3(x, W1) + b1)
    h2 = gelu32(mm3(h1, W2) + b2)
    return ((mm3(h2, W3) + b3) * sc[10:]).astype(np.float32)


def test_bf16_rounding_is_nearest_even():
    assert bf16(np.float32(1.0 + 2.0 ** -8)) == 1.0          # tie -> even
    assert bf16(np.float32(1.0 + 3 * 2.0 ** -8)) == 1.0 + 2.0 ** -6
    h, l = split(np.float32(math.pi))
    assert abs(float(h) + float(l) - math.pi) < 2.0 ** -16 * math.pi


def test_split_product_error_bound():
    from incompact3d_gb300 import sgs
    rng = np.random.default_rng(7)
    P = sgs.init_params(7)
    P[640:704] = rng.uniform(-0.5, 0.5, 64)
    P[4800:4864] = rng.uniform(-0.5, 0.5, 64)
    P[5248:5254] = rng.uniform(-0.5, 0.5, 6)
    sc = np.concatenate([rng.uniform(0.5, 2, 10), rng.uniform(0.5, 2, 6)]).astype(np.float32)
    X = rng.standard_normal((2000, 10)).astype(np.float32)
    ref = np_forward(P.astype(np.float64), sc.astype(np.float64), X.astype(np.float64))[-1] * sc[10:]
    y = tc_forward(P, sc, X)
    err = np.abs(y - ref).max() / np.abs(ref).max()
    assert err < 1e-4, err
    # a plain BF16 product (hi parts only) would not meet it
    W = P[704:4800].reshape(64, 64)
    h = np.abs(np.random.default_rng(1).standard_normal((64, 64))).astype(np.float32)
    one = bf16(h) @ bf16(W).T
    assert np.abs(one - h @ W.T).max() > 1e-4 * np.abs(h @ W.T).max()
