"""Fused momentum term of one direction (x3d_conv_diff_f32) against the same
sum formed from the library's FP64 line operators:
    out = nu d_jj u_q + a1 - (d_j(u_j u_q) + u_j d_j u_q) / 2
(src/transeq.f90:73-591, skew-symmetric convection + viscous term).  The
fused kernel runs in binary32 with its own chunking of the line, so the bar is
binary32 round-off of smooth fields: 2e-5 of the largest value."""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu
L = 2 * np.pi
NU = 1.0 / 1600.0


def smooth(torch, shape, seed):
    """sum of 12 random Fourier modes with |k| <= 6, shape (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z = torch.arange(nz, dtype=torch.float64, device="cuda")[:, None, None] * (L / nz)
    y = torch.arange(ny, dtype=torch.float64, device="cuda")[None, :, None] * (L / ny)
    x = torch.arange(nx, dtype=torch.float64, device="cuda")[None, None, :] * (L / nx)
    f = torch.zeros(shape, dtype=torch.float64, device="cuda")
    for _ in range(12):
        k = rng.integers(-6, 7, size=3)
        f += rng.uniform(0.2, 1.0) * torch.cos(float(k[0]) * x + float(k[1]) * y + float(k[2]) * z
                                                + rng.uniform(0, 2 * np.pi))
    return f


def reference(ctx, gpu_lib, axis, q, uj, uq, a1):
    pu = 0 if q == axis else 1
    A = ctx.apply(axis, gpu_lib.OP_DER1, 1 - pu, (uj * uq).contiguous())
    B = ctx.apply(axis, gpu_lib.OP_DER1, pu, uq)
    C = ctx.apply(axis, gpu_lib.OP_DER2, pu, uq)
    return NU * C + a1 - 0.5 * (A + uj * B)


# (nx, ny, nz): x lines of 128/256/512 run one warp per line, y/z lines of
# 128/256/512 the 16-chunk block kernel
@pytest.mark.parametrize("dims", [(128, 128, 128), (256, 256, 256), (512, 512, 512), (512, 256, 128),
                                  (128, 512, 256)])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_conv_diff_matches_fp64_line_operators(gpu_lib, dims, axis):
    import torch
    nx, ny, nz = dims
    shape = (nz, ny, nx)
    ctx = gpu_lib.Context(nx, ny, nz, L, L, L)
    u = [smooth(torch, shape, 10 + i) for i in range(3)]
    a1 = smooth(torch, shape, 20)
    for q in range(3):
        ref = reference(ctx, gpu_lib, axis, q, u[axis], u[q], a1)
        u32 = [t.float() for t in u]
        out = ctx.conv_diff(axis, q, u32[axis], u32[q], a1.float(), NU)
        assert relerr(out.cpu().numpy(), ref.cpu().numpy()) < 2e-5, (dims, axis, q)
        # without the running sum
        out0 = ctx.conv_diff(axis, q, u32[axis], u32[q], None, NU)
        ref0 = ref - a1
        assert relerr(out0.cpu().numpy(), ref0.cpu().numpy()) < 2e-5, (dims, axis, q)
        # a1 may alias out (the solver accumulates in place)
        acc = a1.float().contiguous()
        ctx.conv_diff(axis, q, u32[axis], u32[q], acc, NU, out=acc)
        assert torch.equal(acc, out)


def test_conv_diff_is_refused_where_the_fused_kernel_does_not_apply(gpu_lib):
    import torch
    from incompact3d_gb300._lib import X3DError
    ctx = gpu_lib.Context(96, 96, 96, L, L, L)  # 96 / 16 = 6 rows per chunk
    u = torch.zeros((96, 96, 96), dtype=torch.float32, device="cuda")
    with pytest.raises(X3DError):
        ctx.conv_diff(1, 0, u, u, None, NU)


# ---- staggered divergence / gradient in binary32 ---------------------------
# divergence: the y and z sums are fused into the circulant solves; gradp: the
# z and y pairs on one input.  Against the FP64 operators on the same (binary32
# representable) inputs.  The FP32 chains differentiate binary32-rounded
# intermediates (e.g. deryvp(interxvp(uy))), which amplifies their rounding by
# about pi/dx, so the bound grows with n: divergence 5e-5 of the largest value
# at n = 128, linear in n; gradient 7e-5 at n = 128, as n^1.5 (the x component
# differentiates two interpolated intermediates).  The 96^3 case runs the
# generic binary32 kernels and sits at the same level.
@pytest.mark.parametrize("dims", [(128, 128, 128), (256, 256, 256), (512, 512, 512), (512, 256, 128),
                                  (128, 512, 256), (96, 96, 96)])
def test_divergence_and_gradp_f32_match_fp64(gpu_lib, dims):
    import torch
    nx, ny, nz = dims
    shape = (nz, ny, nx)
    ctx = gpu_lib.Context(nx, ny, nz, L, L, L)
    u = [smooth(torch, shape, 30 + i).float() for i in range(3)]
    tol = 5e-5 * max(dims) / 128
    tolg = 7e-5 * (max(dims) / 128) ** 1.5
    ref = ctx.divergence(*[t.double() for t in u])
    div = ctx.divergence(*u)
    assert relerr(div.cpu().numpy(), ref.cpu().numpy()) < tol, dims
    p = smooth(torch, shape, 40).float()
    gref = ctx.gradp(p.double())
    g = ctx.gradp(p)
    for a, b in zip(g, gref):
        assert a.dtype == torch.float32
        assert relerr(a.cpu().numpy(), b.cpu().numpy()) < tolg, dims
