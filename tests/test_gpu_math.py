"""Accuracy of the library's own device arithmetic, through the C ABI.

The native FP64 kernels use an FP64 exponential of their own (FP64 argument
reduction, e^r - 1 in double-float on the FP32 pipe, one FP64 FMA to finish);
it stays within 3 ulp of numpy's exp. The double-float kernels' exp,
reciprocal square root, reciprocal and quotient stay within 2^-44 relative
(double-float carries about 48 bits). The float <-> double conversions built
from integer operations (which keep conversions off GB300's FP64 pipe) are
exact, or keep the top 24 bits, as documented.
"""
import numpy as np
import pytest

from mole_gb300 import api

pytestmark = pytest.mark.gpu


def test_fp64_exp_within_3_ulp(ctx):
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.uniform(-60.0, 5.0, 200000), rng.uniform(-699.0, 699.0, 50000),
                        np.linspace(-1.0, 1.0, 20001), [0.0, -0.0, 1e-300, -1e-300, 709.0, -745.0, 800.0, -800.0]])
    y = ctx.math_check(0, x)
    with np.errstate(over="ignore"):
        ref = np.exp(x)
    fin = np.isfinite(ref) & (ref > 0)
    ulps = np.abs(y[fin] - ref[fin]) / np.spacing(ref[fin])
    assert ulps.max() <= 3.0, ulps.max()
    assert np.array_equal(np.isfinite(y), np.isfinite(ref))


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
