"""Accuracy of the library's own device arithmetic, through the C ABI.

The native FP64 kernels use an FP64 exponential of their own (FP64 argument
reduction, e^r - 1 in double-float on the FP32 pipe, one FP64 FMA to finish);
it stays within 3 ulp of numpy's exp. The double-float kernels' exp,
reciprocal square root, reciprocal and quotient stay within 2^-44 relative
(double-float carries about 48 bits).
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
