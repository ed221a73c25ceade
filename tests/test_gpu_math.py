"""Accuracy of the library's own device arithmetic, through the C ABI.

The native FP64 kernels use an FP64 exponential, reciprocal and reciprocal
square root of their own, two FP64-pipe instructions each (the FP32 hardware
approximation, one FP64 FMA correction, integer-built exact doubles; the
exponential reduces by ln2/64 and evaluates e^r - 1 in double-float): the
exponential stays within 2 ulp of numpy's exp, the reciprocal and the
reciprocal square root within 1 ulp of the exact values. The double-float kernels' exp,
reciprocal square root, reciprocal and quotient stay within 2^-44 relative
(double-float carries about 48 bits). The float <-> double conversions built
from integer operations (which keep conversions off GB300's FP64 pipe) are
exact, or keep the top 24 bits, as documented.
"""
import numpy as np
import pytest

from mole_gb300 import api

pytestmark = pytest.mark.gpu


def test_fp64_exp_within_2_ulp(ctx):
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.uniform(-60.0, 5.0, 200000), rng.uniform(-699.0, 699.0, 50000),
                        np.linspace(-1.0, 1.0, 20001), [0.0, -0.0, 1e-300, -1e-300, 709.0, -745.0, 800.0, -800.0]])
    y = ctx.math_check(0, x)
    with np.errstate(over="ignore"):
        ref = np.exp(x)
    fin = np.isfinite(ref) & (ref > 0)
    ulps = np.abs(y[fin] - ref[fin]) / np.spacing(ref[fin])
    assert ulps.max() <= 2.0, ulps.max()
    assert np.array_equal(np.isfinite(y), np.isfinite(ref))


def _exact_ulps(y, x, rsqrt=False):
    """|y - 1/x| (or |y - x^-1/2|) in ulps, the exact value from rational
    arithmetic (for the square root through |1 - x y^2| |y| / 2)."""
    from fractions import Fraction
    out = []
    for yi, xi in zip(y, x):
        xf, yf = Fraction(float(xi)), Fraction(float(yi))
        err = abs(1 - xf * yf * yf) * abs(yf) / 2 if rsqrt else abs(yf - 1 / xf)
        out.append(float(err) / float(np.spacing(abs(float(yi)))))
    return np.array(out)


def test_fp64_reciprocal_within_1_ulp(ctx):
    rng = np.random.default_rng(21)
    x = np.concatenate([rng.uniform(1.0, 2.0, 4000), np.exp(rng.uniform(-40.0, 40.0, 4000)),
                        -np.exp(rng.uniform(-40.0, 40.0, 2000)),
                        [1.0, 2.0, 0.5, 3.0, 1.0 + 2.0 ** -52, 2.0 - 2.0 ** -52]])
    y = ctx.math_check(8, x)
    ulps = _exact_ulps(y, x)
    assert ulps.max() <= 1.0, ulps.max()
    # outside the fast path: the IEEE quotient
    z = np.array([0.0, -0.0, np.inf, -np.inf, 1e-300, 1e300, 2.0 ** -70, 2.0 ** 70])
    with np.errstate(divide="ignore", over="ignore"):
        np.testing.assert_array_equal(ctx.math_check(8, z), 1.0 / z)


def test_fp64_rsqrt_within_1_ulp(ctx):
    rng = np.random.default_rng(22)
    x = np.concatenate([rng.uniform(1.0, 4.0, 4000), np.exp(rng.uniform(-40.0, 40.0, 6000)),
                        [1.0, 2.0, 4.0, 0.25, 1.0 + 2.0 ** -52, 4.0 - 2.0 ** -50]])
    y = ctx.math_check(9, x)
    ulps = _exact_ulps(y, x, rsqrt=True)
    assert ulps.max() <= 1.0, ulps.max()
    z = np.array([0.0, np.inf, 1e-300, 1e300, 2.0 ** -70, 2.0 ** 70])
    with np.errstate(divide="ignore"):
        ref = 1.0 / np.sqrt(z)
    np.testing.assert_allclose(ctx.math_check(9, z), ref, rtol=2e-16)


@pytest.mark.parametrize("fn,lo,hi,kind", [(1, -60.0, 5.0, "uniform"), (2, 1e-10, 1e10, "log"), (3, -1e3, 1e3, "uniform"),
                                           (4, -50.0, 50.0, "uniform")])
def test_double_float_functions_within_2_pow_44(ctx, fn, lo, hi, kind):
    rng = np.random.default_rng(fn)
    x = np.exp(rng.uniform(np.log(lo), np.log(hi), 100000)) if kind == "log" else rng.uniform(lo, hi, 100000)
    x = x[np.abs(x) > 1e-6]
    # the argument as the double-float kernels hold it (48 bits)
    h = x.astype(np.float32).astype(np.float64)
    xd = h + (x - h).astype(np.float32).astype(np.float64)
    ref = {1: np.exp, 2: lambda v: 1.0 / np.sqrt(v), 3: lambda v: 1.0 / v, 4: lambda v: v / (1.0 + x * x)}[fn](xd)
    y = ctx.math_check(fn, x)
    rel = np.abs(y - ref) / np.abs(ref)
    assert rel.max() < 2.0 ** -44, rel.max()


def test_integer_built_conversions(ctx):
    """f2d is exact for normal floats, zeros, infinities and NaNs (subnormals
    become signed zeros); d2f_rz keeps the top 24 bits (rounds toward zero)
    inside FP32's normal range, flushes below it and saturates to infinity
    above it."""
    rng = np.random.default_rng(17)
    x = np.concatenate([rng.normal(0.0, 1.0, 20000) * 10.0 ** rng.integers(-30, 30, 20000),
                        [0.0, -0.0, 1.0, -1.0, 3.4e38, -3.4e38, 1e-39, -1e-39, 1e-300, 1e300, np.inf, -np.inf, np.nan]])
    y = ctx.math_check(5, x)
    with np.errstate(over="ignore"):
        f = x.astype(np.float32)
    ref = np.where(np.abs(f) < np.finfo(np.float32).tiny, np.copysign(0.0, f), f).astype(np.float64)
    fin = ~np.isnan(x)
    np.testing.assert_array_equal(y[fin], ref[fin])
    np.testing.assert_array_equal(np.signbit(y[fin]), np.signbit(ref[fin]))
    assert np.isnan(y[~fin]).all()
    z = ctx.math_check(6, x)
    assert np.isnan(z[~fin]).all()
    z, xf = z[fin], x[fin]
    tiny, big = float(np.finfo(np.float32).tiny), float(np.finfo(np.float32).max)
    normal = (np.abs(xf) >= tiny) & (np.abs(xf) <= big)
    zn, xn = z[normal], xf[normal]
    assert np.array_equal(zn.astype(np.float32).astype(np.float64), zn)  # representable in FP32
    assert np.all(np.abs(zn) <= np.abs(xn)) and np.all(np.sign(zn) == np.sign(xn))
    assert np.all(np.abs(xn - zn) < np.spacing(np.abs(zn).astype(np.float32)).astype(np.float64))
    assert np.all(z[np.abs(xf) < tiny] == 0.0)
    assert np.all(np.isinf(z[np.abs(xf) > big]))
    # the variant for positions agrees wherever its input is below FP32's largest
    small = np.abs(xf) <= big
    np.testing.assert_array_equal(ctx.math_check(7, xf[small]), z[small])
