"""The integer-built pieces of the native FP64 reciprocal, reciprocal square
root, exponential and box proposal (mole_gb300/csrc/fp64.cuh), compiled for
the host and compared with exact rational arithmetic: the sum of a
normalised float pair as a double (exact when it fits 53 bits, a nearest
double otherwise; the power-of-two case where the sum drops a binade), the
split of a double into its top 24 bits and the rounded rest, n L1 for every
reduction index n, and u - 1/2 for 32-bit uniforms."""
import ctypes
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpp", "fp64_host.cu")
OUT = os.path.join(HERE, "cpp", "_build")


@pytest.fixture(scope="module")
def lib():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libfp64_host.so")
    hdrs = [os.path.join(HERE, "..", "mole_gb300", "csrc", h) for h in ("fp64.cuh", "df64.cuh", "common.cuh")]
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(f) for f in [SRC] + hdrs):
        subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                               "-shared", "-Xcompiler", "-fPIC", SRC, "-o", so + ".tmp"])
        os.replace(so + ".tmp", so)
    return ctypes.CDLL(so)


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def nearest(o: float, q: Fraction) -> bool:
    """o is a double nearest to q (a tie may go either way)."""
    return abs(Fraction(o) - q) <= abs(Fraction(float(q)) - q)


def test_dbl_add_small_matches_exact_sum(lib):
    rng = np.random.default_rng(1)
    n = 20000
    h = (rng.uniform(1.0, 2.0, n) * 2.0 ** rng.integers(-60, 60, n)).astype(np.float32)
    h *= np.where(rng.random(n) < 0.3, -1, 1).astype(np.float32)
    # powers of two, with l of both signs (the binade below when opposite)
    h[:2000] = (2.0 ** rng.integers(-60, 60, 2000)).astype(np.float32) * np.where(rng.random(2000) < 0.5, -1, 1)
    ulp = np.spacing(np.abs(h)).astype(np.float64)
    frac = rng.uniform(-0.5, 0.5, n)
    frac[2000:2200] = 0.5
    frac[2200:2400] = -0.5
    l = (frac * ulp * 2.0 ** -rng.integers(0, 30, n)).astype(np.float32)
    l[:50] = 0.0
    out = np.empty(n)
    lib.t_dbl_add_small(P(h), P(l), P(out), n)
    for hi, lo, o in zip(h, l, out):
        assert nearest(float(o), Fraction(float(hi)) + Fraction(float(lo))), (hi, lo, o)


def test_dbl_add_small_exact_products(lib):
    """y^2 = s + se (s the rounded product, se its FMA remainder) is exact."""
    rng = np.random.default_rng(2)
    y = (rng.uniform(1.0, 2.0, 5000) * 2.0 ** rng.integers(-30, 30, 5000)).astype(np.float32)
    s = (y.astype(np.float64) ** 2).astype(np.float32)
    se = np.array([float(Fraction(float(a)) ** 2 - Fraction(float(b))) for a, b in zip(y, s)]).astype(np.float32)
    out = np.empty(y.size)
    lib.t_dbl_add_small(P(s), P(se), P(out), y.size)
    for a, o in zip(y, out):
        assert Fraction(float(o)) == Fraction(float(a)) ** 2


def test_split_double(lib):
    rng = np.random.default_rng(3)
    d = rng.uniform(-1.0, 1.0, 20000) * 2.0 ** rng.integers(-90, 90, 20000)
    d[:3] = [0.0, -0.0, 1e-35]
    h = np.empty(d.size, np.float32)
    l = np.empty(d.size, np.float32)
    lib.t_split_double(P(d), P(h), P(l), d.size)
    for x, a, b in zip(d, h, l):
        if abs(x) < 2.0 ** -100:  # below the split's range: both pieces zero
            assert a == 0 and b == 0
            continue
        m, e = np.frexp(x)  # h: x truncated to 24 significant bits
        assert float(a) == np.ldexp(np.trunc(m * 2.0 ** 24), e - 24)
        rest = Fraction(float(x)) - Fraction(float(a))
        assert abs(Fraction(float(b)) - rest) <= abs(rest) * Fraction(1, 2 ** 24)


def test_exp_nl1_exact_for_every_index(lib):
    k = np.arange(-65535, 65536, dtype=np.int32)
    out = np.empty(k.size)
    lib.t_exp_nl1(P(k), P(out), k.size)
    L1 = Fraction(0xB17217F7D, 2 ** 42)
    assert float(L1) == float.fromhex("0x1.62e42fefap-7")
    for kk in list(range(-65535, -65000)) + list(range(-600, 600)) + list(range(65000, 65536)):
        assert Fraction(float(out[kk + 65535])) == kk * L1
    np.testing.assert_array_equal(out, k.astype(np.float64) * float(L1))  # exact products


def test_u01_centered(lib):
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.integers(0, 2 ** 32, 20000, dtype=np.uint64), [0, 1, 2 ** 31 - 1, 2 ** 31, 2 ** 32 - 1]])
    x = x.astype(np.uint32)
    out = np.empty(x.size)
    lib.t_u01_centered(P(x), P(out), x.size)
    ref = (x.astype(np.float64) + 0.5) * 2.0 ** -32 - 0.5  # exact in double
    np.testing.assert_array_equal(out, ref)
