"""CPU check of the circulant form that the fast periodic kernels use (the
fused momentum and staggered kernels, and the generic kernel's periodic
branch), without a GPU.

A periodic compact system I + alpha (S + S^-1) is solved as
(I + mu S)(I + mu S^-1) / (1 + mu^2): two first-order recurrences run
chunk-locally, joined by cyclic carries with the chunk multiplier (-mu)^L
(incompact3d_gb300.emulate.line_circ replays it in binary64).  For every
operator and parity the library marks circulant (x3d_plan_info), the replay
reproduces the oracle's Thomas + Sherman-Morrison solve
(src/derive.f90 derx_00 and the staggered periodic branches) to round-off,
for warp-style (L = n/32) and block-style (L = 8) chunking.  Plans the
library does not mark circulant (their periodic corners are not those of a
circulant, e.g. the CFP6 p set) do not match it: that is why the kernels
check the flag."""
import numpy as np
import pytest

from conftest import fourier_field, relerr


@pytest.fixture(scope="module")
def x3d():
    import incompact3d_gb300 as m
    m.build()
    return m


@pytest.mark.parametrize("n,L", [(64, 8), (128, 4), (128, 8), (256, 8)])
@pytest.mark.parametrize("kind", range(7))
@pytest.mark.parametrize("npaire", [0, 1])
def test_circulant_replay_matches_oracle(x3d, oracle_mod, kind, npaire, n, L):
    from incompact3d_gb300 import emulate
    Ls = (2 * np.pi, 2.0, 3.0)
    dims = (n, 8, 8)
    ctx = x3d.Context(*dims, *Ls, filter_alpha=0.45)
    o = oracle_mod.Oracle(*dims, *Ls, filter_alpha=0.45)
    p = emulate.plan(ctx, 0, kind, npaire)
    u = fourier_field(*dims, L=Ls, seed=kind + 7 * npaire + n)
    ref = o.op(0, kind, npaire, u)
    got = emulate.line_circ(kind, p, u, L)
    if p["circulant"]:
        assert relerr(got, ref) < 1e-13, (kind, npaire, n, L)
    else:
        assert relerr(got, ref) > 1e-8, (kind, npaire, n, L)


def test_every_centred_operator_is_circulant(x3d):
    """First and second derivatives and the filter are circulant for both
    parities on a periodic axis (the momentum right-hand side relies on it)."""
    from incompact3d_gb300 import emulate
    ctx = x3d.Context(128, 8, 8, 2 * np.pi, 2.0, 3.0)
    for kind in (0, 1, 2):
        for npaire in (0, 1):
            assert emulate.plan(ctx, 0, kind, npaire)["circulant"], (kind, npaire)


def test_carry_count_follows_the_chunk_multiplier(x3d):
    from incompact3d_gb300 import emulate
    ctx = x3d.Context(128, 8, 8, 2 * np.pi, 2.0, 3.0)
    p = emulate.plan(ctx, 0, 0, 1)
    mu, A, J = emulate.circ_coefs(p, 8)
    assert 0 < mu < 0.5 and A == pytest.approx(mu ** 8)
    assert abs(A) ** J < 2.0 ** -60 <= abs(A) ** (J - 1)
    assert emulate.circ_coefs(p, 4)[2] > J  # shorter chunks, weaker damping, more carries
