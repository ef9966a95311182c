"""GPU parity of every compact operator against the CPU oracle.

Each operator (first/second derivative, filter, the four staggered operators)
along x, y and z, for every boundary-condition pair and parity the reference
implements (src/derive.f90, src/filters.f90), in FP64 and FP32, called through
the C ABI.  Tolerances, relative to the field's max: FP64 1e-12 (the parity
bound); FP32 1e-4 (binary32 round-off amplified by the one-sided Dirichlet
closures of the second derivative, whose coefficients are O(10/dx^2)).
"""
import numpy as np
import pytest

from conftest import fourier_field, relerr

pytestmark = pytest.mark.gpu

OPS = ["der1", "der2", "fil", "dvp", "ivp", "dpv", "ipv"]
BCS = [(0, 0), (1, 1), (2, 2), (1, 2), (2, 1)]
TOL = {"float64": 1e-12, "float32": 1e-4}


def _cases():
    out = []
    for kind in range(7):
        for bc in BCS:
            for npaire in (0, 1):
                if bc != (0, 0) and npaire == 0 and kind in (4, 5, 6):
                    continue  # no such branch in the reference
                if bc == (0, 0) and npaire == 0 and kind in (3, 4, 5, 6):
                    continue  # parity is irrelevant for periodic staggered ops
                out.append((kind, bc, npaire))
    return out


def _make(oracle_mod, gpu_lib, dims, axis, bc):
    bcs = [(0, 0), (0, 0), (0, 0)]
    bcs[axis] = bc
    Ls = (2 * np.pi, 2.0, 3.0)
    ctx = gpu_lib.Context(*dims, *Ls, bc=tuple(bcs), filter_alpha=0.45)
    o = oracle_mod.Oracle(*dims, *Ls, bc=tuple(bcs), filter_alpha=0.45)
    return ctx, o, Ls, bcs


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("kind,bc,npaire", _cases())
def test_operator_matches_oracle(oracle_mod, gpu_lib, kind, bc, npaire, axis, dtype):
    import torch
    dims = [37, 22, 19]
    ctx, o, Ls, bcs = _make(oracle_mod, gpu_lib, dims, axis, bc)
    per = [b == (0, 0) for b in bcs]
    shp = list(dims)
    if kind in (5, 6):  # p->v: input on the pressure mesh along the axis
        shp[axis] = ctx.nm[axis]
    u = fourier_field(*shp, L=Ls, seed=7 + kind, periodic=per)
    ref = o.op(axis, kind, npaire, u)
    tdt = getattr(torch, dtype)
    ud = torch.from_numpy(u).to(device="cuda", dtype=tdt)
    out = ctx.apply(axis, kind, npaire, ud)
    torch.cuda.synchronize()
    got = out.double().cpu().numpy()
    assert got.shape == ref.shape
    assert relerr(got, ref) < TOL[dtype], (OPS[kind], bc, npaire, axis, dtype, relerr(got, ref))


@pytest.mark.parametrize("n", [8, 16, 64, 128, 512])
def test_line_lengths(oracle_mod, gpu_lib, n):
    """Chunking edge cases: lines shorter than, equal to and longer than the 16 chunks."""
    import torch
    L = 2 * np.pi
    for bc in [(0, 0), (2, 2)]:
        dims = (n, 9, 8)
        ctx = gpu_lib.Context(*dims, L, L, L, bc=(bc, (0, 0), (0, 0)))
        o = oracle_mod.Oracle(*dims, L, L, L, bc=(bc, (0, 0), (0, 0)))
        u = fourier_field(*dims, seed=n, periodic=(bc == (0, 0), True, True))
        for kind in (0, 1, 2):
            ref = o.op(0, kind, 0, u)
            got = ctx.apply(0, kind, 0, torch.from_numpy(u).cuda()).cpu().numpy()
            assert relerr(got, ref) < 1e-12, (n, bc, kind)


def test_reference_signatures_and_coefficient_sets(oracle_mod, gpu_lib):
    """derx/dery/.../filz with the coefficient vectors the reference passes."""
    import torch
    n = (32, 24, 20)
    L = 2 * np.pi
    bc = ((2, 2), (1, 1), (0, 0))
    ctx = gpu_lib.Context(*n, L, L, L, bc=bc)
    o = oracle_mod.Oracle(*n, L, L, L, bc=bc)
    u = fourier_field(*n, seed=3, periodic=(False, False, True))
    ud = torch.from_numpy(u).cuda()
    t = torch.empty_like(ud)
    for npaire, sfx in ((0, ""), (1, "P")):
        ctx.derx(t, ud, None, None, ctx.coeffs(0, "FF" + sfx), ctx.coeffs(0, "FS" + sfx), ctx.coeffs(0, "FW" + sfx),
                 *n, npaire=npaire)
        assert relerr(t.cpu().numpy(), o.op(0, 0, npaire, u)) < 1e-12
        ctx.dery(t, ud, None, None, ctx.coeffs(1, "FF" + sfx), ctx.coeffs(1, "FS" + sfx), ctx.coeffs(1, "FW" + sfx),
                 None, *n, npaire=npaire)
        assert relerr(t.cpu().numpy(), o.op(1, 0, npaire, u)) < 1e-12
        ctx.derzz(t, ud, None, None, ctx.coeffs(2, "SF" + sfx), ctx.coeffs(2, "SS" + sfx), ctx.coeffs(2, "SW" + sfx),
                  *n, npaire=npaire)
        assert relerr(t.cpu().numpy(), o.op(2, 1, npaire, u)) < 1e-12
        ctx.fily(t, ud, None, None, ctx.coeffs(1, "FIFF" + sfx), ctx.coeffs(1, "FIFS" + sfx),
                 ctx.coeffs(1, "FIFW" + sfx), *n, npaire=npaire)
        assert relerr(t.cpu().numpy(), o.op(1, 2, npaire, u)) < 1e-12
    # a coefficient vector that is not one of the context's sets is refused
    bad = ctx.coeffs(0, "FF") * 1.0000001
    with pytest.raises(gpu_lib.X3DError) as e:
        ctx.derx(t, ud, None, None, bad, ctx.coeffs(0, "FS"), ctx.coeffs(0, "FW"), *n, npaire=0)
    assert e.value.status == -6
    # wrong extents
    with pytest.raises(gpu_lib.X3DError) as e:
        ctx.derx(t, ud, nx=31, ny=24, nz=20)
    assert e.value.status == -2


def test_full_size_512_sampled_lines(oracle_mod, gpu_lib):
    """512^3 operators (the microbench size) checked on sampled lines: lines are
    independent, so the oracle runs on a thin slab holding whole lines."""
    import torch
    n = 512
    L = 2 * np.pi
    ctx = gpu_lib.Context(n, n, n, L, L, L)
    o = oracle_mod.Oracle(n, n, n, L, L, L)
    rng = np.random.default_rng(11)
    u = torch.randn((n, n, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(5))
    for kind in (0, 1, 2, 3, 4):
        for axis in range(3):
            out = ctx.apply(axis, kind, 1, u)
            torch.cuda.synchronize()
            a, b = rng.integers(0, n - 2, size=2)
            if axis == 0:
                ui, go = u[a:a + 2, b:b + 2, :], out[a:a + 2, b:b + 2, :]
            elif axis == 1:
                ui, go = u[a:a + 2, :, b:b + 2], out[a:a + 2, :, b:b + 2]
            else:
                ui, go = u[:, a:a + 2, b:b + 2], out[:, a:a + 2, b:b + 2]
            ref = o.op(axis, kind, 1, ui.contiguous().cpu().numpy())
            assert relerr(go.cpu().numpy(), ref) < 1e-12, (kind, axis)
    del u
    torch.cuda.empty_cache()


@pytest.mark.parametrize("n", [128, 256, 512])
def test_fp32_fast_path_periodic(oracle_mod, gpu_lib, n):
    """FP32 periodic lines of 16*L points (L = 8, 16, 32) run the register-window
    fast path (line_fast); every operator kind on every axis vs the oracle."""
    import torch
    L = 2 * np.pi
    for axis in range(3):
        dims = [24, 20, 18]
        dims[axis] = n
        ctx = gpu_lib.Context(*dims, L, L, L, filter_alpha=0.45)
        o = oracle_mod.Oracle(*dims, L, L, L, filter_alpha=0.45)
        u = fourier_field(*dims, seed=n + axis, kmax=6)
        ud = torch.from_numpy(u).to(device="cuda", dtype=torch.float32)
        for kind in range(7):
            ref = o.op(axis, kind, 1, u)
            got = ctx.apply(axis, kind, 1, ud).double().cpu().numpy()
            # binary32 round-off of the second difference grows like (n/(2 pi k))^2
            tol = 1e-4 * max(1.0, (n / 256.0) ** 2) if kind == 1 else 1e-4
            assert relerr(got, ref) < tol, (n, axis, OPS[kind], relerr(got, ref))
