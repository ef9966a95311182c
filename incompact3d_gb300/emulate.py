"""Exact numpy model of the line kernel's arithmetic (x3d_line_kernel.cuh),
driven by the host plan the library exports (x3d_plan_info).

Used by the CPU tests to check, without a GPU, that the plan tables (boundary
rows, chunked-solve fix-up factors, Sherman-Morrison vector) reproduce the
oracle.  It follows the kernel step by step: right-hand side per row, chunk-
local forward sweep, carry scan, fix-up, chunk-local back substitution, carry
scan, fix-up, periodic correction.
"""
import ctypes

import numpy as np

from . import _lib

KMAXB, KMAXT, KMAXE = 10, 6, 4
BROW = 2 + KMAXT * (2 + 2 * KMAXE)


def plan(ctx, axis, op, npaire, coefset=-1):
    lib = _lib.load()
    sc = np.zeros(16)
    vec = np.zeros(6 * 4096)
    br = np.zeros(KMAXB * BROW)
    n = _lib.check(lib.x3d_plan_info(ctx.h, axis, op, npaire, coefset, sc.ctypes.data_as(ctypes.c_void_p),
                                     vec.ctypes.data_as(ctypes.c_void_p), br.ctypes.data_as(ctypes.c_void_p)),
                   "x3d_plan_info")
    p = dict(nin=int(sc[0]), nout=int(sc[1]), L=int(sc[2]), periodic=bool(sc[3]), ca=sc[4], cb=sc[5],
             cc=sc[6], cd=sc[7], alpha=sc[8], den=sc[9], nbrows=int(sc[10]), nterms=int(sc[11]),
             chunks=int(sc[12]), circulant=bool(sc[13]))
    for q, name in enumerate(("s", "f", "w", "pf", "qb", "rsm")):
        p[name] = vec[q * n:(q + 1) * n].copy()
    rows = {}
    for q in range(p["nbrows"]):
        o = br[q * BROW:(q + 1) * BROW]
        terms = []
        for t in range(int(o[1])):
            ot = o[2 + t * (2 + 2 * KMAXE):2 + (t + 1) * (2 + 2 * KMAXE)]
            ents = [(int(ot[2 + 2 * e]), int(ot[3 + 2 * e])) for e in range(int(ot[1]))]
            terms.append((ot[0], ents))
        rows[int(o[0])] = terms
    p["brows"] = rows
    return p


def _interior(op, U, r, p):
    ca, cb, cc, cd = p["ca"], p["cb"], p["cc"], p["cd"]
    if op == 0:
        return ca * (U(r + 1) - U(r - 1)) + cb * (U(r + 2) - U(r - 2))
    if op == 1:
        ur = U(r)
        acc = ca * (U(r + 1) - ur - ur + U(r - 1)) + cb * (U(r + 2) - ur - ur + U(r - 2))
        if p["nterms"] > 2:
            acc = acc + cc * (U(r + 3) - ur - ur + U(r - 3)) + cd * (U(r + 4) - ur - ur + U(r - 4))
        return acc
    if op == 2:
        return ca * U(r) + cb * (U(r + 1) + U(r - 1)) + cc * (U(r + 2) + U(r - 2)) + cd * (U(r + 3) + U(r - 3))
    if op == 3:
        return ca * (U(r + 1) - U(r)) + cb * (U(r + 2) - U(r - 1))
    if op == 4:
        acc = ca * (U(r + 1) + U(r)) + cb * (U(r + 2) + U(r - 1)) + cc * (U(r + 3) + U(r - 2))
        if p["nterms"] > 3:
            acc = acc + cd * (U(r + 4) + U(r - 3))
        return acc
    if op == 5:
        return ca * (U(r) - U(r - 1)) + cb * (U(r + 1) - U(r - 2))
    acc = ca * (U(r) + U(r - 1)) + cb * (U(r + 1) + U(r - 2)) + cc * (U(r + 2) + U(r - 3))
    if p["nterms"] > 3:
        acc = acc + cd * (U(r + 3) + U(r - 4))
    return acc


EXT = {0: (-2, 2), 1: (-4, 4), 2: (-3, 3), 3: (-1, 2), 4: (-3, 4), 5: (-2, 1), 6: (-4, 3)}


def line(op, p, u):
    """Apply the kernel's arithmetic to a batch of lines u[..., nin]."""
    nin, nout, L, C = p["nin"], p["nout"], p["L"], p["chunks"]
    lo, hi = EXT[op]
    t = np.zeros(u.shape[:-1] + (nout,))
    for r in range(nout):
        if r + lo >= 0 and r + hi < nin:
            t[..., r] = _interior(op, lambda i: u[..., i], r, p)
        elif p["periodic"]:
            t[..., r] = _interior(op, lambda i: u[..., i % nin], r, p)
        else:
            acc = None
            for coef, ents in p["brows"].get(r, []):
                v = ents[0][1] * u[..., ents[0][0]]
                for idx, mult in ents[1:]:
                    v = v + mult * u[..., idx]
                acc = coef * v if acc is None else acc + coef * v
            t[..., r] = 0.0 if acc is None else acc
    s, f, w, pf, qb = p["s"], p["f"], p["w"], p["pf"], p["qb"]
    chunks = [(c * L, min(c * L + L, nout)) for c in range(C) if c * L < nout]
    # forward, chunk-local
    ends = []
    for r0, r1 in chunks:
        y = np.zeros(u.shape[:-1])
        for r in range(r0, r1):
            y = t[..., r] - s[r] * y
            t[..., r] = y
        ends.append(y.copy())
    cin = np.zeros(u.shape[:-1])
    for ci, (r0, r1) in enumerate(chunks):
        if ci > 0:
            for r in range(r0, r1):
                t[..., r] = t[..., r] + pf[r] * cin
        cin = t[..., r1 - 1].copy()
    # backward, chunk-local
    starts = []
    for r0, r1 in chunks:
        x = np.zeros(u.shape[:-1])
        for r in range(r1 - 1, r0 - 1, -1):
            x = (t[..., r] - f[r] * x) * w[r]
            t[..., r] = x
        starts.append(x.copy())
    cin = np.zeros(u.shape[:-1])
    for ci in range(len(chunks) - 1, -1, -1):
        r0, r1 = chunks[ci]
        if ci < len(chunks) - 1:
            for r in range(r0, r1):
                t[..., r] = t[..., r] + qb[r] * cin
        cin = t[..., r0].copy()
    if p["periodic"]:
        sx = (t[..., 0] - p["alpha"] * t[..., nout - 1]) / p["den"]
        t = t - sx[..., None] * p["rsm"]
    return t


def circ_coefs(p, L, lim=2.0 ** -60, max_carries=64):
    """Circulant form of a periodic plan for chunks of L rows: the factor mu of
    I + alpha (S + S^-1) = (I + mu S)(I + mu S^-1) / (1 + mu^2), the chunk
    multiplier A = (-mu)^L and the number J of cyclic carries kept (the
    weights |A|^(j-1) above lim), as the host fills them for the kernels."""
    al = p["alpha"]
    mu = 2.0 * al / (1.0 + np.sqrt(1.0 - 4.0 * al * al))
    A = (-mu) ** L
    J = 1
    w = abs(A)
    while J < max_carries and w >= lim:
        J += 1
        w *= abs(A)
    return mu, A, J


def line_circ(op, p, u, L, lim=2.0 ** -60):
    """The circulant-form solve of the fast kernels (x3d_circ.cuh and the
    generic kernel's periodic branch) on a batch of periodic lines
    u[..., n], n a multiple of L: right-hand side with coefficients scaled by
    1 + mu^2, chunk-local forward recurrence z_i = b_i - mu z_(i-1), cyclic
    carries between chunks (J terms), fix-up (-mu)^(k+1) * carry; the same
    backwards with x_i = z_i - mu x_(i+1) and (-mu)^(L-k)."""
    n = p["nout"]
    if n % L or not p["periodic"]:
        raise ValueError("line_circ: periodic lines of a multiple of L rows only")
    mu, A, J = circ_coefs(p, L, lim)
    sc = 1.0 + mu * mu
    ps = dict(p, ca=p["ca"] * sc, cb=p["cb"] * sc, cc=p["cc"] * sc, cd=p["cd"] * sc)
    C = n // L
    t = np.stack([_interior(op, lambda i: u[..., i % n], r, ps) for r in range(n)], axis=-1)
    t = t.reshape(u.shape[:-1] + (C, L))
    for k in range(L):  # forward, chunk-local
        if k:
            t[..., k] = t[..., k] - mu * t[..., k - 1]
    end = t[..., L - 1].copy()
    carry = np.zeros_like(end)
    for j in range(1, J + 1):
        carry += A ** (j - 1) * np.roll(end, j, axis=-1)
    pw = (-mu) ** (np.arange(L) + 1)
    t += carry[..., None] * pw
    for k in range(L - 2, -1, -1):  # backward, chunk-local
        t[..., k] = t[..., k] - mu * t[..., k + 1]
    start = t[..., 0].copy()
    # the backward pass above ran on the fixed-up z; its carries come from the
    # chunk starts to the right
    carry = np.zeros_like(start)
    for j in range(1, J + 1):
        carry += A ** (j - 1) * np.roll(start, -j, axis=-1)
    qw = (-mu) ** (L - np.arange(L))
    t += carry[..., None] * qw
    return t.reshape(u.shape[:-1] + (n,))


def apply(ctx, axis, op, npaire, u, coefset=-1):
    """Operator along `axis` of a (nz, ny, nx) numpy field, kernel arithmetic."""
    p = plan(ctx, axis, op, npaire, coefset)
    ax = 2 - axis
    v = np.moveaxis(u, ax, -1)
    return np.moveaxis(line(op, p, v), -1, ax)
