"""kg_math.h on the device (sm_103a) against the host build: identical bits.

The kernels and the CPU oracle share these functions as source; this checks
that nvcc's device build (no FMA contraction, correctly rounded FP32 seed)
computes the same bits as the host build, on random and edge-case inputs, and
that the constant-divisor path equals the GPU's own IEEE division.
"""
import ctypes
import math

import numpy as np
import pytest

import ko_oracle
from crystalgrowth_gb300 import _lib

pytestmark = pytest.mark.gpu


def dev_eval(fn, x, b=1.0):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    _lib.check(_lib.lib().kg_diag_eval(fn, _lib.dptr(x), _lib.dptr(y), x.size, float(b)))
    return y


def inputs(seed, n=2_000_000):
    rng = np.random.default_rng(seed)
    edge = np.array([0.0, -0.0, 1.0, -1.0, 5e-324, -5e-324, 2.0 ** -1022, 2.0 ** -900, 2.0 ** -899, 2.0 ** 899,
                     2.0 ** 64, 2.0 ** 65, 1e300, math.inf, -math.inf, math.nan, 4095.99, -4095.99, 4096.0,
                     math.pi / 2, math.pi, 1 + 2 ** -52, 1 - 2 ** -53])
    with np.errstate(over="ignore"):  # magnitudes above 1e308 become infinities on purpose
        wide = rng.standard_normal(n) * 10.0 ** rng.integers(-310, 310, n)
    return np.concatenate([edge, rng.uniform(-2, 2, n), rng.uniform(-70, 70, n), wide, rng.uniform(9, 11, n // 4)])


def same_bits(a, b):
    return np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("fn", [0, 1, 2])
def test_transcendentals_device_equals_host(fn):
    x = inputs(100 + fn)
    assert same_bits(dev_eval(fn, x), ko_oracle.kg_eval(fn, x))


@pytest.mark.parametrize("b", [0.03, 3 * 0.03 * 0.03, 3e-4, 2.1e-4, 3.99e-4, 1e-4, 9e-4, 7.0, 1 / 3, 0.5, 2.0 ** -99])
def test_constant_division_equals_ieee_on_device(b):
    rng = np.random.default_rng(int(b * 1e7) % 991)
    k = rng.integers(1, 53, 500_000)
    sub = ((rng.integers(0, 2 ** 62, k.size, dtype=np.int64) % (2 ** k)) | 1).astype(np.float64) * 5e-324
    x = np.concatenate([inputs(int(b * 1e7) % 997), sub, -sub])
    ieee = dev_eval(4, x, b)
    assert same_bits(dev_eval(5, x, b), ieee)
    assert same_bits(ieee, ko_oracle.kg_eval(4, x, b))


def test_fp64_peak_probe():
    v = ctypes.c_double()
    _lib.check(_lib.lib().kg_diag_fp64_peak(ctypes.byref(v)))
    assert v.value > 1e10


def test_twice_plus_equals_two_roundings_on_device():
    """kg_twice_plus(x, y) (one FMA, integer finish where 2 x overflows) == RN(RN(2 x) + y) on the device,
    including |x| >= 2^1023, infinities and NaN"""
    rng = np.random.default_rng(78)
    n = 2_000_000
    big = rng.uniform(1, 2, n) * 2.0 ** 1023 * rng.choice([-1, 1], n)
    cases = [rng.standard_normal(n) * 10.0 ** rng.integers(-320, 308, n),
             np.concatenate([rng.uniform(-1, 1, n), -2 * rng.uniform(-1, 1, n)[::-1]]),
             np.concatenate([big, rng.standard_normal(n) * 10.0 ** rng.integers(300, 308, n)]),
             np.concatenate([big[:8], [math.inf, -math.inf, math.nan, -1.7976931348623157e308, 1.7976931348623157e308,
                                       0.0, -0.0, 5e-324]]),
             np.array([2.0 ** 1023, 1.5 * 2.0 ** 1023, -2.0 ** 1023, math.inf, -math.inf, math.nan, 1.0,
                       -math.inf, math.inf, -1.7976931348623157e308, math.inf, -math.inf])]
    for x in cases:
        with np.errstate(all="ignore"):
            a, r = dev_eval(10, x), dev_eval(11, x)
            assert (((a.view(np.uint64) == r.view(np.uint64)) | (np.isnan(a) & np.isnan(r))).all())


def test_gdiv_equals_ieee_division_on_device():
    """kg_gdiv(x[i], x[n-1-i]) on the device has the bits of the GPU's own IEEE division, subnormal
    operands and quotients included"""
    rng = np.random.default_rng(79)
    n = 2_000_000
    a = rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n)
    near = np.concatenate([1 + rng.integers(0, 2 ** 20, n) * 2.0 ** -52, 2 - rng.integers(1, 2 ** 20, n) * 2.0 ** -52])
    m = rng.uniform(1, 2, n)
    edge = np.array([0.0, -0.0, 1.0, -1.0, 3.0, 2.0 ** -1022, 5e-324, -5e-324, 1.7976931348623157e308,
                     2.0 ** 1000, 2.0 ** -1000, math.inf, -math.inf, math.nan, 0.1, 1e-300, 1e300, 7.0])
    cases = [np.concatenate([a, a[::-1] * rng.uniform(0.5, 2, n)]), near * rng.choice([-1, 1], 2 * n),
             np.concatenate([m, m[::-1]]),
             np.concatenate([rng.uniform(1, 2, n) * 2.0 ** 1000, rng.uniform(1, 2, n) * 2.0 ** -30]),
             np.concatenate([rng.uniform(1, 2, n) * 2.0 ** -1000, rng.uniform(1, 2, n) * 2.0 ** 30]),
             np.concatenate([edge, np.resize(edge[::-1], edge.size)])]
    k = rng.integers(1, 53, n)
    sub = ((rng.integers(0, 2 ** 62, n, dtype=np.int64) % (2 ** k)) | 1).astype(np.float64) * 5e-324
    cases += [np.concatenate([sub, rng.uniform(0.01, 100, n)]), np.concatenate([sub, sub[::-1]]),
              np.concatenate([rng.uniform(1, 2, n) * 2.0 ** rng.integers(-1060, -1000, n), sub[::-1]])]
    for x in cases:
        with np.errstate(all="ignore"):
            a_, r_ = dev_eval(13, x), dev_eval(14, x)
            assert (((a_.view(np.uint64) == r_.view(np.uint64)) | (np.isnan(a_) & np.isnan(r_))).all())
