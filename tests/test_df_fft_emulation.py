"""CPU replay of the double-float (binary32 hi + lo) butterfly arithmetic of
the Poisson FFT (csrc/x3d_fft.cu): the radix-8 butterfly with unnormalised
inner sums and the complex product that folds all error terms into one lo
sum.  Against a long-double DFT the replayed butterfly stays within a few
2^-48 of the inputs' size, no worse than the fully renormalised form, and
the folded complex product within 2^-45 of |a||b| (its single lo sum takes
more binary32 roundings than four renormalised products: about 1.5x their
error, still a few units of 2^-48).

binary32 arithmetic is numpy's (round to nearest); a fused multiply-add is
replayed as an exact binary64 product plus one sum, which matches the
hardware except for rare double roundings in the last bit of a lo part."""
import numpy as np
import pytest

f32 = np.float32
LD = np.longdouble
U48 = 2.0 ** -48


def fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def two_sum(a, b):
    s = a + b
    v = s - a
    return s, (a - (s - v)) + (b - v)


def fast_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def add(a, b):
    sh, sl = two_sum(a[0], b[0])
    return fast_two_sum(sh, sl + (a[1] + b[1]))


def add_l(a, b):  # lazy: no renormalisation
    sh, sl = two_sum(a[0], b[0])
    return sh, sl + (a[1] + b[1])


def neg(a):
    return -a[0], -a[1]


def mul(a, b):
    p = a[0] * b[0]
    e = fma(a[0], b[0], -p)
    e = fma(a[0], b[1], e)
    e = fma(a[1], b[0], e)
    return fast_two_sum(p, e)


def dot2(x, y, u, v, sg):
    uh, ul = (u[0], u[1]) if sg > 0 else (-u[0], -u[1])
    p1 = x[0] * y[0]
    p2 = uh * v[0]
    e1 = fma(x[0], y[0], -p1)
    e2 = fma(uh, v[0], -p2)
    sh, sl = two_sum(p1, p2)
    t = sl + (e1 + e2)
    t = fma(x[0], y[1], t)
    t = fma(x[1], y[0], t)
    t = fma(uh, v[1], t)
    t = fma(ul, v[0], t)
    return fast_two_sum(sh, t)


# complex double-float: (re, im), each a (hi, lo) pair of binary32 arrays
def cadd(a, b, lazy):
    f = add_l if lazy else add
    return f(a[0], b[0]), f(a[1], b[1])


def csub(a, b, lazy):
    f = add_l if lazy else add
    return f(a[0], neg(b[0])), f(a[1], neg(b[1]))


def cmul_folded(a, b):
    return dot2(a[0], b[0], a[1], b[1], -1), dot2(a[0], b[1], a[1], b[0], 1)


def cmul_plain(a, b):
    return (add(mul(a[0], b[0]), neg(mul(a[1], b[1]))), add(mul(a[0], b[1]), mul(a[1], b[0])))


def mul_i(a, s):
    return (a[1], neg(a[0])) if s < 0 else (neg(a[1]), a[0])


H = (f32(0.70710677), f32(1.2101617e-08))


def w8_1(o, s, lazy):
    x, y = o
    f = add_l if lazy else add
    if s < 0:
        return mul(f(x, y), H), mul(f(y, neg(x)), H)
    return mul(f(x, neg(y)), H), mul(f(y, x), H)


def w8_3(o, s, lazy):
    x, y = o
    f = add_l if lazy else add
    if s < 0:
        return mul(f(y, neg(x)), H), neg(mul(f(x, y), H))
    return neg(mul(f(x, y), H)), mul(f(x, neg(y)), H)


def fft4(x, s, inner, lazy):
    s02, d02 = cadd(x[0], x[2], lazy), csub(x[0], x[2], lazy)
    s13, d13 = cadd(x[1], x[3], lazy), mul_i(csub(x[1], x[3], lazy), s)
    last = lazy and inner
    return [cadd(s02, s13, last), cadd(d02, d13, last), csub(s02, s13, last), csub(d02, d13, last)]


def fft8(v, s, lazy=True):
    e = fft4([v[0], v[2], v[4], v[6]], s, True, lazy)
    o = fft4([v[1], v[3], v[5], v[7]], s, True, lazy)
    t = [o[0], w8_1(o[1], s, lazy), mul_i(o[2], s), w8_3(o[3], s, lazy)]
    return [cadd(e[k], t[k], False) for k in range(4)] + [csub(e[k], t[k], False) for k in range(4)]


def split(x):
    h = x.astype(f32)
    return h, (x - h.astype(np.float64)).astype(f32)


def value(p):
    return p[0].astype(LD) + p[1].astype(LD)


def rand_cdf(rng, n, scale=1.0):
    return split(rng.standard_normal(n) * scale), split(rng.standard_normal(n) * scale)


@pytest.mark.parametrize("sign", [-1, 1])
def test_radix8_butterfly_with_lazy_inner_sums(sign):
    rng = np.random.default_rng(8 + sign)
    n = 20000
    # magnitudes spread over 2^-10 .. 2^10 between the 8 inputs of a butterfly
    v = [rand_cdf(rng, n, 2.0 ** rng.integers(-10, 11)) for _ in range(8)]
    xr = np.stack([value(a[0]) for a in v])
    xi = np.stack([value(a[1]) for a in v])
    j = np.arange(8, dtype=LD)
    ang = sign * 2 * np.pi * np.outer(j, j) / LD(8)
    c, s = np.cos(ang), np.sin(ang)
    Xr = c @ xr - s @ xi
    Xi = s @ xr + c @ xi
    norm = np.sqrt((xr ** 2 + xi ** 2).sum(0))
    errs = {}
    for lazy in (True, False):
        out = fft8(v, sign, lazy)
        er = np.stack([value(o[0]) for o in out]) - Xr
        ei = np.stack([value(o[1]) for o in out]) - Xi
        errs[lazy] = float(np.max(np.sqrt(er ** 2 + ei ** 2) / norm))
    assert errs[True] < 8 * U48, errs
    assert errs[True] < 2.0 * errs[False] + U48, errs


def test_folded_complex_product():
    rng = np.random.default_rng(3)
    n = 50000
    a = rand_cdf(rng, n)
    b = rand_cdf(rng, n)
    ar, ai, br, bi = (value(a[0]), value(a[1]), value(b[0]), value(b[1]))
    exact_r, exact_i = ar * br - ai * bi, ar * bi + ai * br
    scale = np.sqrt(ar ** 2 + ai ** 2) * np.sqrt(br ** 2 + bi ** 2)
    errs = {}
    for f in (cmul_folded, cmul_plain):
        r = f(a, b)
        err = np.sqrt((value(r[0]) - exact_r) ** 2 + (value(r[1]) - exact_i) ** 2) / scale
        errs[f.__name__] = float(err.max())
    assert errs["cmul_folded"] < 8 * U48, errs
    assert errs["cmul_plain"] < 8 * U48, errs
    assert errs["cmul_folded"] < 2.0 * errs["cmul_plain"], errs
