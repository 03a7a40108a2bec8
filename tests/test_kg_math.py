"""kg_math.h (host build): faithful atan / sin / cos, and the integer-pipe divisions == IEEE division.

These functions are shared source between the CUDA kernels and the CPU
oracle; the GPU tests check the device build against the same values.
"""
import math

import numpy as np
import pytest

import ko_oracle

mp = pytest.importorskip("mpmath")
mp.mp.prec = 200


def ulp_err(got, exact):
    e = float(exact)
    if e == 0.0:
        return 0.0 if got == 0.0 else math.inf
    return float(abs(mp.mpf(got) - exact) / math.ulp(e))


def test_atan_faithful_random():
    """the integer-pipe atan: faithful everywhere, and within 0.55 ulp (nearly always correctly
    rounded: its fixed-point error is below 2^-55 relative) on every branch -- the table (t in
    [2^-7, 1]), the small-t series, and the reciprocal for |x| > 1 (including |x| >= 128)"""
    rng = np.random.default_rng(11)
    xs = np.concatenate([rng.uniform(-1, 1, 3000), rng.uniform(-20, 20, 3000),
                         10.0 ** rng.uniform(-12, 12, 3000) * rng.choice([-1, 1], 3000),
                         rng.uniform(9.5, 10.5, 1000), 1.0 + rng.uniform(-1e-9, 1e-9, 500),
                         rng.uniform(2.0 ** -8, 2.0 ** -6, 500), rng.uniform(120, 140, 500),
                         2.0 ** rng.integers(-27, 64, 300).astype(float),
                         (np.arange(1, 129) / 128.0) * (1 + rng.uniform(-1e-15, 1e-15, 128))])
    worst = max(ulp_err(ko_oracle.kg_atan(x), mp.atan(mp.mpf(float(x)))) for x in xs)
    assert worst < 0.55


def test_atan_special_values():
    a = ko_oracle.kg_atan
    assert a(0.0) == 0.0 and math.copysign(1, a(0.0)) == 1
    assert a(-0.0) == 0.0 and math.copysign(1, a(-0.0)) == -1
    assert a(math.inf) == math.pi / 2 and a(-math.inf) == -math.pi / 2
    assert math.isnan(a(math.nan))
    assert a(1e300) == math.pi / 2
    assert a(1.0) == math.atan(1.0)
    assert a(-1.0) == -math.atan(1.0)
    assert a(5e-324) == 5e-324
    for x in (0.5, 2.0, 10.0, 1e-8, 123.0):
        assert a(-x) == -a(x)


def test_sincos_accuracy_random():
    """the integer-pipe sin/cos (|x| < 64): absolute error below 2^-61 everywhere, faithful (< 1 ulp)
    wherever |value| >= 2^-9; near a zero of sin or cos the absolute bound is what holds (the step
    only ever adds these values to O(1) quantities).  |x| >= 64 (never reached by the step, whose
    argument j (theta - theta0) stays below 64) takes the FP64 formulation: about 1 ulp."""
    rng = np.random.default_rng(12)
    xs = np.concatenate([rng.uniform(-60, 60, 5000), rng.uniform(-64, 64, 1000), rng.uniform(-1e-3, 1e-3, 500),
                         rng.uniform(-2.0 ** -5, 2.0 ** -5, 500), 2.0 ** rng.uniform(-27, -5, 500),
                         np.arange(-64, 65) * (math.pi / 128), np.arange(-20, 21) * (math.pi / 2)])
    worst_abs = worst_ulp = 0.0
    for x in xs:
        s, c = ko_oracle.kg_sincos(x)
        for got, ex in ((s, mp.sin(mp.mpf(float(x)))), (c, mp.cos(mp.mpf(float(x))))):
            worst_abs = max(worst_abs, float(abs(mp.mpf(got) - ex)) - math.ulp(float(ex)) / 2)
            if abs(float(ex)) >= 2.0 ** -9:
                worst_ulp = max(worst_ulp, ulp_err(got, ex))
    assert worst_abs < 2.0 ** -61 and worst_ulp < 1.0
    big = np.concatenate([rng.uniform(-4000, -64, 500), rng.uniform(64, 4000, 500)])
    ws = wc = 0.0
    for x in big:
        s, c = ko_oracle.kg_sincos(x)
        ws = max(ws, ulp_err(s, mp.sin(mp.mpf(float(x)))))
        wc = max(wc, ulp_err(c, mp.cos(mp.mpf(float(x)))))
    assert ws < 1.25 and wc < 1.25


def test_sincos_small_arguments_keep_relative_precision():
    """|x| in [2^-27, 2^-5): sin x keeps x's relative precision (faithful), cos x is faithful"""
    rng = np.random.default_rng(14)
    for x in 2.0 ** rng.uniform(-27, -5, 2000) * rng.choice([-1, 1], 2000):
        s, c = ko_oracle.kg_sincos(x)
        assert ulp_err(s, mp.sin(mp.mpf(float(x)))) < 1.0 and ulp_err(c, mp.cos(mp.mpf(float(x)))) < 1.0
        assert math.copysign(1, s) == math.copysign(1, x)


def test_sincos_domain():
    s, c = ko_oracle.kg_sincos(0.0)
    assert s == 0.0 and c == 1.0
    for x in (4096.0, -4096.0, 1e10, math.inf, math.nan):
        s, c = ko_oracle.kg_sincos(x)
        assert math.isnan(s) and math.isnan(c)


@pytest.mark.parametrize("b", [0.03, 3 * 0.03 * 0.03, 3e-4, 2.1e-4, 1e-4, 7.0, 1 / 3, 0.5, 1.0, 0.75, 2.0 ** -99,
                               2.0 ** 99])
def test_idiv_matches_ieee_random(b):
    """kg_idiv (integer significand division) == IEEE a / b, including zeros, subnormals,
    infinities, NaN and quotients that underflow or overflow"""
    rng = np.random.default_rng(int(b * 1e6) % 1000 + 7)
    n = 1_000_000
    x = np.concatenate([rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n), rng.uniform(-1, 1, n),
                        rng.integers(2 ** 52, 2 ** 53, n).astype(np.float64) * 2.0 ** rng.integers(-1074, 970, n),
                        np.array([0.0, -0.0, 5e-324, -5e-324, 2.0 ** -1022, math.inf, -math.inf, 1e308, -1e308,
                                  2.0 ** -1000, math.nan])])
    with np.errstate(all="ignore"):
        ref = x / b
    got = ko_oracle.kg_eval(5, x, b)
    same = (got.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(got) & np.isnan(ref))
    assert same.all()


def _pairs(seed, n=1_000_000):
    rng = np.random.default_rng(seed)
    base = rng.standard_normal(n)
    sub = rng.integers(0, 2 ** 53, n).astype(np.float64) * 5e-324 * rng.choice([-1, 1], n)
    edge = np.array([0.0, -0.0, 5e-324, -5e-324, 1.7976931348623157e308, 1.7976931348623157e308, -0.0, -0.0,
                     math.inf, -math.inf, math.nan, 1.0, 2.0 ** -1022, -2.0 ** -1022, 1e308, 1e308])
    return [rng.standard_normal(n) * 10.0 ** rng.integers(-320, 308, n),
            np.concatenate([base, -base[::-1] * (1 + rng.integers(-50, 50, n) * 2.0 ** -52)]),
            np.concatenate([rng.uniform(-1, 1, n), rng.uniform(-1, 1, n) * 2.0 ** rng.integers(-60, 60, n)]),
            np.concatenate([sub, sub * rng.uniform(0, 3, n)]), edge]


def _same(a, r):
    return bool(((a.view(np.uint64) == r.view(np.uint64)) | (np.isnan(a) & np.isnan(r))).all())


def test_twice_plus_equals_two_roundings():
    """kg_twice_plus(x, y) == RN(RN(2 x) + y): one FMA where 2 x is exact, integers where it overflows"""
    rng = np.random.default_rng(23)
    n = 1_000_000
    big = rng.uniform(1, 2, n) * 2.0 ** 1023 * rng.choice([-1, 1], n)
    cases = _pairs(24) + [np.concatenate([big, rng.standard_normal(n) * 10.0 ** rng.integers(300, 308, n)]),
                          np.array([2.0 ** 1023, -2.0 ** 1023, 1.5 * 2.0 ** 1023, math.inf, -math.inf, math.nan,
                                    -math.inf, math.inf, -1.7976931348623157e308, 1.0, math.nan, -math.inf])]
    for x in cases:
        with np.errstate(all="ignore"):
            assert _same(ko_oracle.kg_eval(10, x), ko_oracle.kg_eval(11, x))


def test_absorb_bound():
    """kg_absorb_bound(c): every |t| up to it leaves c - t == c (both signs of t and c), and it is
    2^(e-55) for normal c in [2^e, 2^(e+1)); zero, subnormal and non-finite c give 0 (only t = +-0)"""
    rng = np.random.default_rng(25)
    c = np.concatenate([rng.uniform(0.5, 1.5, 20000), rng.uniform(-4, 4, 20000),
                        rng.standard_normal(20000) * 10.0 ** rng.integers(-307, 307, 20000),
                        [1.0, 2.0, 0.5, 2.0 ** -1022, 2.0 ** -1000, 2.0 ** -968, 2.0 ** -967, 1.7976931348623157e308,
                         0.0, -0.0, 5e-324, math.inf, math.nan]])
    bound = ko_oracle.kg_eval(12, c)
    fin = np.isfinite(c) & (np.abs(c) >= 2.0 ** -1022)
    assert not bound[~fin].any()
    e = np.frexp(np.abs(c[fin]))[1] - 1  # c in [2^e, 2^(e+1))
    with np.errstate(under="ignore"):
        want = np.ldexp(1.0, (e - 55).astype(np.int64))
    assert np.array_equal(bound[fin], want)
    for s in (1.0, -1.0):
        for f in (1.0, 0.999, 0.5, 2.0 ** -20):
            t = s * bound * f
            with np.errstate(all="ignore"):
                ok = np.where(np.isfinite(c), c - t, c)
            assert np.array_equal(ok[np.isfinite(c)], c[np.isfinite(c)])


def _div_pairs(seed, n=1_000_000):
    """dividend/divisor pairs (x[i], x[n-1-i]): wide exponents, significands near 1 and 2, equal
    significands, powers of two, results near the overflow and underflow limits, specials"""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n)
    near1 = 1 + rng.integers(0, 2 ** 20, n) * 2.0 ** -52
    near2 = 2 - rng.integers(1, 2 ** 20, n) * 2.0 ** -52
    m = rng.uniform(1, 2, n)
    edge = np.array([0.0, -0.0, 1.0, -1.0, 3.0, 2.0 ** -1022, 5e-324, -5e-324, 1.7976931348623157e308,
                     2.0 ** 1000, 2.0 ** -1000, math.inf, -math.inf, math.nan, 0.1, 1e-300, 1e300, 7.0])
    return [np.concatenate([a, a[::-1] * rng.uniform(0.5, 2, n)]),
            np.concatenate([near1 * rng.choice([-1, 1], n), near2[::-1] * 2.0 ** rng.integers(-8, 8, n)]),
            np.concatenate([m, m[::-1]]),                                   # equal significands
            np.concatenate([m * 2.0 ** rng.integers(-60, 60, n), 2.0 ** rng.integers(-30, 30, n)]),
            np.concatenate([rng.uniform(1, 2, n) * 2.0 ** 1000, rng.uniform(1, 2, n) * 2.0 ** -30]),   # overflow
            np.concatenate([rng.uniform(1, 2, n) * 2.0 ** -1000, rng.uniform(1, 2, n) * 2.0 ** 30]),   # underflow
            np.concatenate([edge, edge[::-1] * 0 + np.resize(edge, edge.size)])]


def test_gdiv_matches_ieee_division():
    """kg_gdiv(x[i], x[n-1-i]) has the bits of the IEEE quotient (the oracle's own '/')"""
    for seed in (31, 32):
        for x in _div_pairs(seed):
            with np.errstate(all="ignore"):
                assert _same(ko_oracle.kg_eval(13, x), ko_oracle.kg_eval(14, x))


def test_gdiv_every_significand_pair_small_grid():
    """every dividend significand against every divisor significand on a 2^-9 grid of [1, 2), and
    the 2^12 divisor significands nearest each power of two"""
    g = 1 + np.arange(512) * 2.0 ** -9
    a = np.repeat(g, g.size)
    b = np.tile(g, g.size)
    x = np.concatenate([a, b[::-1]])
    with np.errstate(all="ignore"):
        assert _same(ko_oracle.kg_eval(13, x), ko_oracle.kg_eval(14, x))
    rng = np.random.default_rng(33)
    d = np.concatenate([1 + np.arange(1, 4097) * 2.0 ** -52, 2 - np.arange(1, 4097) * 2.0 ** -52])
    a = rng.uniform(1, 2, d.size)
    x = np.concatenate([a, d[::-1]])
    with np.errstate(all="ignore"):
        assert _same(ko_oracle.kg_eval(13, x), ko_oracle.kg_eval(14, x))


def _subnormals(rng, n):
    """every subnormal magnitude scale: random significand bits below 2^k, k = 1..52, both signs"""
    k = rng.integers(1, 53, n)
    m = (rng.integers(0, 2 ** 62, n, dtype=np.int64) % (2 ** k)).astype(np.int64) | 1
    return (m.astype(np.float64) * 5e-324) * rng.choice([-1, 1], n)


@pytest.mark.parametrize("b", [0.03, 3 * 0.03 * 0.03, 3e-4, 2.1e-4, 7.0, 1 / 3, 0.5, 2.0 ** -99, 2.0 ** 99, 1e-4])
def test_idiv_subnormal_dividends(b):
    """subnormal dividends (normalised on the integer pipes) and subnormal quotients (rounded once from
    the exact remainder) have the bits of the IEEE division"""
    rng = np.random.default_rng(int(b * 1e7) % 977 + 3)
    x = np.concatenate([_subnormals(rng, 1_000_000), rng.uniform(1, 2, 200_000) * 2.0 ** rng.integers(-1080, -1000, 200_000)])
    with np.errstate(all="ignore"):
        ref = x / b
    assert _same(ko_oracle.kg_eval(5, x, b), ref)


def test_gdiv_subnormal_operands_and_results():
    """kg_gdiv with subnormal dividends, subnormal divisors, and quotients in the subnormal range
    (every rounding position) has the bits of the IEEE division"""
    rng = np.random.default_rng(35)
    n = 1_000_000
    sub = _subnormals(rng, n)
    cases = [np.concatenate([sub, rng.uniform(0.01, 100, n)]),                       # subnormal / normal
             np.concatenate([rng.uniform(1, 2, n) * 2.0 ** rng.integers(-1060, -1000, n), sub[::-1]]),   # / subnormal
             np.concatenate([rng.uniform(1, 2, n) * 2.0 ** rng.integers(-1022, -960, n),
                             rng.uniform(1, 2, n) * 2.0 ** rng.integers(1, 110, n)]),  # normal / normal -> subnormal
             np.concatenate([sub, sub[::-1]])]
    for x in cases:
        with np.errstate(all="ignore"):
            assert _same(ko_oracle.kg_eval(13, x), ko_oracle.kg_eval(14, x))
