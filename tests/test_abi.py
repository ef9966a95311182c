"""The C ABI without a GPU: the library loads, exports every symbol that
include/x3d_gpu.h declares, builds its host-side tables, and its coefficient
vectors are bit-identical to the oracle's restatement of src/schemes.f90 and
src/filters.f90.  Host-side argument checks return the documented statuses.
No compute call is made here."""
import ctypes

import numpy as np
import pytest

L = 2 * np.pi


@pytest.fixture(scope="module")
def lib():
    import incompact3d_gb300 as x3d
    x3d.build()
    return x3d


def test_exports_every_declared_symbol(lib):
    from incompact3d_gb300 import _lib
    so = _lib.load()
    names = _lib.declared_symbols()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(so, n)]
    assert missing == []


CASES = [((0, 0), (0, 0), (0, 0)), ((2, 2), (1, 1), (1, 2)), ((2, 1), (2, 2), (1, 1)), ((1, 1), (0, 0), (2, 2))]


@pytest.mark.parametrize("bc", CASES)
@pytest.mark.parametrize("opts", [dict(), dict(isecondder=5, ipinter=2, filter_alpha=0.3), dict(ipinter=1)])
def test_coefficients_bitwise_equal_oracle(lib, oracle_mod, bc, opts):
    from incompact3d_gb300 import _lib
    dims = (24, 17, 33)
    ctx = lib.Context(*dims, L, 2.0, 3.0, bc=bc, **opts)
    o = oracle_mod.Oracle(*dims, L, 2.0, 3.0, bc=bc, **opts)
    for axis in range(3):
        for w in range(33):
            a = o.coeffs(axis, w)
            b = ctx.coeffs(axis, _lib.COEF_NAMES[w])
            assert a.shape == b.shape, (axis, _lib.COEF_NAMES[w])
            assert np.array_equal(a, b), (axis, _lib.COEF_NAMES[w])


def test_host_side_argument_checks(lib):
    from incompact3d_gb300 import _lib
    so = _lib.load()
    h = ctypes.c_void_p()
    o = _lib.NumOpts(4, 4, 3, 0.49, 4.0, 0.44)
    # mixed periodic / non-periodic ends on one axis
    g = _lib.Grid(16, 16, 16, L, L, L, 0, 2, 0, 0, 0, 0, 0, 0.0)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)) == -3
    # stretching needs a non-periodic y (src/parameters.f90:283); istret is 0..3
    g = _lib.Grid(16, 16, 16, L, L, L, 0, 0, 0, 0, 0, 0, 2, 0.259)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)) == -3
    g = _lib.Grid(16, 17, 16, L, L, L, 0, 0, 2, 2, 0, 0, 4, 0.259)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)) == -7
    g = _lib.Grid(16, 17, 16, L, L, L, 0, 0, 2, 2, 0, 0, 2, 0.259)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)) == 0
    so.x3d_ctx_destroy(h)
    # too small
    g = _lib.Grid(4, 16, 16, L, L, L, 0, 0, 0, 0, 0, 0, 0, 0.0)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)) == -2
    # unsupported scheme
    g = _lib.Grid(16, 16, 16, L, L, L, 0, 0, 0, 0, 0, 0, 0, 0.0)
    bad = _lib.NumOpts(2, 4, 3, 0.49, 4.0, 0.44)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(bad), ctypes.byref(h)) == -7
    assert so.x3d_ctx_create(None, ctypes.byref(o), ctypes.byref(h)) == -1
    assert so.x3d_strerror(-6) == b"coefficient vectors match no set of this context"
    # fused momentum term: argument, shape and stretching checks come first
    g = _lib.Grid(16, 16, 16, L, L, L, 0, 0, 0, 0, 0, 0, 0, 0.0)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)) == 0
    p = ctypes.c_void_p(256)  # never dereferenced
    one = ctypes.c_float(1.0)
    assert so.x3d_conv_diff_f32(h, 3, 0, p, p, p, None, one, (ctypes.c_int * 3)(16, 16, 16), None) == -1
    assert so.x3d_conv_diff_f32(h, 0, 3, p, p, p, None, one, (ctypes.c_int * 3)(16, 16, 16), None) == -1
    assert so.x3d_conv_diff_f32(h, 0, 0, p, p, p, None, one, (ctypes.c_int * 3)(16, 16, 8), None) == -2
    so.x3d_ctx_destroy(h)
    g = _lib.Grid(16, 17, 16, L, L, L, 0, 0, 2, 2, 0, 0, 2, 0.259)
    assert so.x3d_ctx_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h)) == 0
    assert so.x3d_conv_diff_f32(h, 1, 0, p, p, p, None, one, (ctypes.c_int * 3)(16, 17, 16), None) == -7
    so.x3d_ctx_destroy(h)
    assert so.x3d_conv_diff_f32(None, 0, 0, p, p, p, None, one, (ctypes.c_int * 3)(16, 16, 16), None) == -1
    # NULL context handles are rejected before any device work
    assert so.x3d_derx(None, None, None, None, None, None, None, None, 16, 16, 16, 0, 0.0, None) == -1
    assert so.x3d_poisson(None, None, None) == -1
    assert so.x3d_solver_step(None, 1, None) == -1
