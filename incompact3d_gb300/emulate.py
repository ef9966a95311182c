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
             chunks=int(sc[12]))
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


def apply(ctx, axis, op, npaire, u, coefset=-1):
    """Operator along `axis` of a (nz, ny, nx) numpy field, kernel arithmetic."""
    p = plan(ctx, axis, op, npaire, coefset)
    ax = 2 - axis
    v = np.moveaxis(u, ax, -1)
    return np.moveaxis(line(op, p, v), -1, ax)
