"""Pins of the CPU oracle against the reference's known answers (no GPU).

* compute_k2 (src/Case-TGV.f90:928-950): the closed-form modified wavenumber of
  the periodic second derivative, and its first-derivative / staggered / filter
  analogues built from the coefficients of src/schemes.f90 and
  src/filters.f90 (waves, src/poisson.f90:1574-1585);
* Dirichlet closures reproduce low-order polynomials exactly;
* the projection of solve_poisson leaves a divergence at round-off level
  (src/navier.f90:257-372, README claim "div u at machine precision");
* TGV invariants: E_k(0) = 1/8, the Re=1600 decay over the first steps;
* the 2-D TGV space-time discrete damping (compute_tgv2D_errors,
  src/Case-TGV.f90:827-924).
"""
import numpy as np
import pytest

from conftest import fourier_field, relerr

L = 2 * np.pi


def test_first_derivative_modified_wavenumber(oracle_mod):
    o = oracle_mod.Oracle(32, 24, 16, L, L, L)
    for axis, n in enumerate((32, 24, 16)):
        s = o.scalars(axis)
        d = s["d"]
        for k in (1, 3, 5):
            x = np.arange(n) * d
            shape = [1, 1, 1]
            shape[2 - axis] = n
            u = np.broadcast_to(np.sin(k * x).reshape(shape), (16, 24, 32)).copy()
            t = o.op(axis, oracle_mod.OP_DER1, 0, u)
            kp = (2 * s["afi"] * np.sin(k * d) + 2 * s["bfi"] * np.sin(2 * k * d)) / (1 + 2 * s["alfai"] * np.cos(k * d))
            ref = np.broadcast_to((kp * np.cos(k * x)).reshape(shape), u.shape)
            assert relerr(t, ref) < 1e-13


def test_second_derivative_compute_k2(oracle_mod):
    # k2 of src/Case-TGV.f90:945-949 (derxx_00 applied to sin(kx) = -k2 sin(kx))
    for isecondder in (4, 5):
        o = oracle_mod.Oracle(64, 16, 16, L, L, L, isecondder=isecondder)
        s = o.scalars(0)
        d = s["d"]
        x = np.arange(64) * d
        for k in (1.0, 4.0, 9.0):
            u = np.broadcast_to(np.sin(k * x), (16, 16, 64)).copy()
            t = o.op(0, oracle_mod.OP_DER2, 0, u)
            k2 = (s["asi"] * 2 * (1 - np.cos(k * d)) + 4 * s["bsi"] * 0.5 * (1 - np.cos(2 * k * d))
                  + 9 * s["csi"] * (2 / 9) * (1 - np.cos(3 * k * d)) + 16 * s["dsi"] * (1 / 8) * (1 - np.cos(4 * k * d)))
            k2 = k2 / (1 + 2 * s["alsai"] * np.cos(k * d))
            assert relerr(t, -k2 * u) < 1e-12


def test_filter_transfer_function(oracle_mod):
    o = oracle_mod.Oracle(48, 16, 16, L, L, L, filter_alpha=0.3)
    s = o.scalars(0)
    d = s["d"]
    x = np.arange(48) * d
    for k in (2, 7, 15):
        u = np.broadcast_to(np.cos(k * x), (16, 16, 48)).copy()
        t = o.op(0, oracle_mod.OP_FIL, 0, u)
        w = k * d
        tf = (s["fiai"] + 2 * s["fibi"] * np.cos(w) + 2 * s["fici"] * np.cos(2 * w) + 2 * s["fidi"] * np.cos(3 * w)) \
            / (1 + 2 * s["fiali"] * np.cos(w))
        assert relerr(t, tf * u) < 1e-13


def test_staggered_modified_wavenumbers(oracle_mod):
    # waves, src/poisson.f90:1574-1585: derivative at mid-points and the
    # interpolation transfer function (src/poisson.f90:1688-1724).
    n = 32
    o = oracle_mod.Oracle(n, 16, 16, L, L, L)
    s = o.scalars(0)
    d = s["d"]
    x = np.arange(n) * d
    xm = x + 0.5 * d
    for k in (1, 4, 9):
        w = k * d
        u = np.broadcast_to(np.sin(k * x), (16, 16, n)).copy()
        t = o.op(0, oracle_mod.OP_DVP, 0, u)
        wp = (2 * s["aci6"] * d * np.sin(w / 2) + 2 * s["bci6"] * d * np.sin(1.5 * w)) / (1 + 2 * s["alcai6"] * np.cos(w))
        assert relerr(t, np.broadcast_to(wp / d * np.cos(k * xm), t.shape)) < 1e-13
        ti = o.op(0, oracle_mod.OP_IVP, 1, u)
        tr = (2 * s["aici6"] * np.cos(w / 2) + 2 * s["bici6"] * np.cos(1.5 * w) + 2 * s["cici6"] * np.cos(2.5 * w)
              + 2 * s["dici6"] * np.cos(3.5 * w)) / (1 + 2 * s["ailcai6"] * np.cos(w))
        assert relerr(ti, np.broadcast_to(tr * np.sin(k * xm), ti.shape)) < 1e-13
        # pressure mesh back to velocity mesh
        p = np.broadcast_to(np.sin(k * xm), (16, 16, n)).copy()
        tp = o.op(0, oracle_mod.OP_DPV, 1, p)
        assert relerr(tp, np.broadcast_to(wp / d * np.cos(k * x), tp.shape)) < 1e-13


@pytest.mark.parametrize("bc", [(2, 2), (1, 2), (2, 1)])
def test_dirichlet_closures_exact_on_polynomials(oracle_mod, bc):
    n = 33
    o = oracle_mod.Oracle(n, 16, 16, 2.0, 1.0, 1.0, bc=(bc, (0, 0), (0, 0)))
    x = np.linspace(0, 2.0, n)
    if bc == (2, 2):
        u = np.broadcast_to(0.3 + 1.7 * x - 0.8 * x ** 2 + 0.25 * x ** 3, (16, 16, n)).copy()
        t = o.op(0, oracle_mod.OP_DER1, 0, u)
        assert relerr(t, np.broadcast_to(1.7 - 1.6 * x + 0.75 * x ** 2, u.shape)) < 1e-12
        u2 = np.broadcast_to(0.3 + 1.7 * x - 0.8 * x ** 2, (16, 16, n)).copy()
        t2 = o.op(0, oracle_mod.OP_DER2, 0, u2)
        assert np.max(np.abs(t2 + 1.6)) < 1e-9
        # the boundary points are not filtered
        tf = o.op(0, oracle_mod.OP_FIL, 0, u)
        assert tf[..., 0] == pytest.approx(u[..., 0], rel=0, abs=0)
        assert tf[..., -1] == pytest.approx(u[..., -1], rel=0, abs=0)
    else:
        # free-slip wall at one end: an even function has zero slope there
        xe = x if bc[0] == 1 else (2.0 - x)
        u = np.broadcast_to(np.cos(np.pi * xe / 4.0), (16, 16, n)).copy()
        t = o.op(0, oracle_mod.OP_DER1, 1, u)
        wall = 0 if bc[0] == 1 else -1
        assert abs(t[..., wall]).max() == 0.0


def test_projection_is_divergence_free(oracle_mod):
    n = 32
    o = oracle_mod.Oracle(n, n, n, L, L, L)
    u = [fourier_field(n, n, n, seed=s) for s in (1, 2, 3)]
    pp3 = o.divergence(*u)
    p = o.poisson(pp3)
    px, py, pz = o.gradp(p)
    v = [u[0] - px, u[1] - py, u[2] - pz]
    dv = o.divergence(*v)
    assert np.abs(dv).max() < 1e-12 * np.abs(pp3).max() + 1e-13


def test_tgv_initial_energy_and_decay(oracle_mod):
    n = 32
    o = oracle_mod.Oracle(n, n, n, L, L, L)
    x = np.arange(n) * L / n
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    ux = np.sin(X) * np.cos(Y) * np.cos(Z)
    uy = -np.cos(X) * np.sin(Y) * np.cos(Z)
    uz = np.zeros_like(ux)
    st = o.tgv_stats(ux, uy, uz, 1 / 1600.0)
    assert st[0] == pytest.approx(0.125, rel=1e-14)
    a, b, c, rows, dmax = o.run(ux, uy, uz, 20, 0.005, 1 / 1600.0, 3, 10)
    assert rows.shape == (2, 5)
    assert np.all(np.diff(rows[:, 1]) < 0)          # kinetic energy decays
    assert rows[0, 1] == pytest.approx(0.125, rel=1e-3)
    assert dmax < 1e-12
    # dE/dt = -eps (energy balance of the semi-discrete system, loose)
    dedt = (rows[1, 1] - rows[0, 1]) / 0.05
    assert dedt == pytest.approx(-rows[:, 2].mean(), rel=0.05)


def _k2(s, k):
    """Modified wavenumber squared of the second derivative (compute_k2,
    src/Case-TGV.f90:928-950)."""
    d = s["d"]
    k2 = (s["asi"] * 2 * (1 - np.cos(k * d)) + 4 * s["bsi"] * 0.5 * (1 - np.cos(2 * k * d))
          + 9 * s["csi"] * (2 / 9) * (1 - np.cos(3 * k * d)) + 16 * s["dsi"] * (1 / 8) * (1 - np.cos(4 * k * d)))
    return k2 / (1 + 2 * s["alsai"] * np.cos(k * d))


def _ab_decay(lam, dt, nsteps):
    """Amplitude of y' = -lam y after nsteps of the AB3 scheme with its Euler
    and AB2 start-up (src/time_integrators.f90:86-100)."""
    a, f = 1.0, []
    for it in range(nsteps):
        f.insert(0, -lam * a)
        if it == 0:
            inc = f[0]
        elif it == 1:
            inc = 1.5 * f[0] - 0.5 * f[1]
        else:
            inc = 23 / 12 * f[0] - 16 / 12 * f[1] + 5 / 12 * f[2]
        a += dt * inc
    return a


@pytest.mark.parametrize("n,nu,dt,nsteps", [(32, 0.1, 0.001, 1), (32, 0.1, 0.001, 50), (64, 0.1, 0.002, 50),
                                            (32, 1 / 1600.0, 0.005, 40)])
def test_tgv2d_space_time_discrete_damping(oracle_mod, n, nu, dt, nsteps):
    """The 2-D TGV check of the reference (compute_tgv2D_errors,
    src/Case-TGV.f90:827-924): u = sin x cos y, v = -cos x sin y stays that
    single mode, its amplitude decays by 1 - 2 k2 dt nu per explicit Euler
    step (the space-time discrete damping, k2 from compute_k2 at k = 1), and
    by the same AB2 / AB3 recurrence on -2 nu k2 after the start-up; the
    analytic exp(-2 nu t) is met to the scheme's truncation error."""
    nz = 8
    o = oracle_mod.Oracle(n, n, nz, L, L, L)
    x = np.arange(n) * L / n
    X, Y = x[None, None, :], x[None, :, None]
    mode = np.sin(X) * np.cos(Y)
    ux = np.broadcast_to(mode, (nz, n, n)).copy()
    uy = np.broadcast_to(-np.cos(X) * np.sin(Y), (nz, n, n)).copy()
    uz = np.zeros((nz, n, n))
    a, b, c, rows, dmax = o.run(ux, uy, uz, nsteps, dt, nu, 3, nsteps)
    amp = float((a * mode).sum() / (mode * mode).sum() / nz)
    lam = 2 * nu * _k2(o.scalars(0), 1.0)
    if nsteps == 1:
        assert abs(amp - (1 - lam * dt)) < 1e-14
    assert abs(amp - _ab_decay(lam, dt, nsteps)) < 1e-13
    assert np.abs(a - amp * mode).max() < 1e-13            # still the single mode
    assert np.abs(b + amp * np.cos(X) * np.sin(Y)).max() < 1e-13
    assert np.abs(c).max() < 1e-13
    assert abs(amp - np.exp(-2 * nu * nsteps * dt)) < 1e-7
