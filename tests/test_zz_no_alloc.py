"""The allocation-free Poisson entry point, x3d_poisson_noalloc.

It serves callers that must not allocate device memory when they solve (their
device memory is reserved up front in their own pool); instead of the
context's lazily allocated spectrum it uses one fixed array in the library's
device image.  This file is collected last on purpose, and is also meant to
pass when run alone in a fresh process.

Checks, through the C ABI: two calls in a row give the same result as
x3d_poisson within the parity tolerance of the other Poisson tests (1e-12
relative), and a grid whose spectrum does not fit the fixed array is refused
with X3D_ERR_SCRATCH without touching the input."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
L = 2 * np.pi


def _noalloc(ctx, t):
    import torch
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return ctx.lib.x3d_poisson_noalloc(ctx.h, ctypes.c_void_p(t.data_ptr()), st)


@pytest.mark.parametrize("dims", [(32, 32, 32), (64, 32, 16), (128, 128, 128)])
def test_noalloc_poisson_matches_x3d_poisson_twice(gpu_lib, dims):
    import torch
    ctx = gpu_lib.Context(*dims, L, 2.0, 3.0)
    g = torch.Generator("cuda").manual_seed(sum(dims))
    rhs = torch.randn((dims[2], dims[1], dims[0]), dtype=torch.float64, device="cuda", generator=g)
    rhs -= rhs.mean()
    ref = rhs.clone()
    ctx.poisson(ref)
    for _ in range(2):
        out = rhs.clone()
        assert _noalloc(ctx, out) == 0
        torch.cuda.synchronize()
        err = (out - ref).abs().max().item() / ref.abs().max().item()
        assert err < 1e-12, err


def test_noalloc_poisson_refuses_grids_beyond_its_scratch(gpu_lib):
    import torch
    n = 256  # spectrum 129*256*256*16 B = 135 MB > 64 MiB
    ctx = gpu_lib.Context(n, n, n, L, L, L)
    rhs = torch.ones((n, n, n), dtype=torch.float64, device="cuda")
    assert _noalloc(ctx, rhs) == -10  # X3D_ERR_SCRATCH
    torch.cuda.synchronize()
    assert rhs.min().item() == 1.0 and rhs.max().item() == 1.0
