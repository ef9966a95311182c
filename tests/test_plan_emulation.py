"""CPU check of the line kernel's plan tables (no GPU).

The library exports each operator's host plan (x3d_plan_info): interior
coefficients, boundary-row table, Thomas factors, chunked-solve fix-up
factors and the Sherman-Morrison vector.  incompact3d_gb300.emulate replays
the kernel's arithmetic on those tables in numpy; it must reproduce the oracle
for every operator, boundary-condition pair and parity."""
import numpy as np
import pytest

from conftest import fourier_field, relerr

BCS = [(0, 0), (1, 1), (2, 2), (1, 2), (2, 1)]


def cases():
    out = []
    for kind in range(7):
        for bc in BCS:
            for npaire in (0, 1):
                if bc != (0, 0) and npaire == 0 and kind in (4, 5, 6):
                    continue
                out.append((kind, bc, npaire))
    return out


@pytest.fixture(scope="module")
def x3d():
    import incompact3d_gb300 as m
    m.build()
    return m


@pytest.mark.parametrize("kind,bc,npaire", cases())
def test_emulated_kernel_matches_oracle(x3d, oracle_mod, kind, bc, npaire):
    from incompact3d_gb300 import emulate
    for axis in range(3):
        dims = [21, 18, 40]
        bcs = [(0, 0)] * 3
        bcs[axis] = bc
        Ls = (2 * np.pi, 2.0, 3.0)
        ctx = x3d.Context(*dims, *Ls, bc=tuple(bcs), filter_alpha=0.45)
        o = oracle_mod.Oracle(*dims, *Ls, bc=tuple(bcs), filter_alpha=0.45)
        shp = list(dims)
        if kind in (5, 6):
            shp[axis] = ctx.nm[axis]
        u = fourier_field(*shp, L=Ls, seed=kind + 3 * axis, periodic=[b == (0, 0) for b in bcs])
        ref = o.op(axis, kind, npaire, u)
        got = emulate.apply(ctx, axis, kind, npaire, u)
        assert relerr(got, ref) < 1e-13, (kind, bc, npaire, axis)


def test_unsupported_parities_are_refused(x3d):
    ctx = x3d.Context(20, 16, 16, 2.0, 1.0, 1.0, bc=((2, 2), (0, 0), (0, 0)))
    from incompact3d_gb300 import emulate
    for kind in (4, 5, 6):
        with pytest.raises(x3d.X3DError) as e:
            emulate.plan(ctx, 0, kind, 0)
        assert e.value.status == -3
