"""The error analysis of the energy series against the reference's formulas
(scripts/statfor.rs, restated in oracle/compat.py) and against AR(1) series
whose autocorrelation time is known: tau = (1 + phi) / (1 - phi)."""
import numpy as np
import pytest

from mole_gb300 import statistics as st
from oracle import compat


def ar1(n, phi, rng):
    x = np.empty(n)
    x[0] = rng.normal()
    e = rng.normal(size=n) * np.sqrt(1.0 - phi * phi)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + e[i]
    return x


@pytest.mark.parametrize("phi", [0.0, 0.5, 0.9])
def test_tau_corr_matches_statfor(phi):
    x = ar1(5000, phi, np.random.default_rng(1))
    a = st.tau_corr(x)
    b = compat.statfor_correlation(x)
    np.testing.assert_allclose(a, b, rtol=1e-10)


@pytest.mark.parametrize("phi", [0.5, 0.8])
def test_tau_corr_of_ar1(phi):
    x = ar1(200000, phi, np.random.default_rng(2))
    tau, _, _ = st.tau_corr(x)
    assert tau == pytest.approx((1 + phi) / (1 - phi), rel=0.1)


def test_blocking_matches_statfor_on_whole_blocks():
    x = ar1(4096, 0.7, np.random.default_rng(3))
    ref = dict(compat.statfor_blocking(x))
    c = st.blocking_curve(x, min_blocks=20)
    for size, err in zip(c.sizes, c.errors):
        if x.size % size == 0 and size in ref:
            assert err == pytest.approx(ref[size], rel=1e-12)


def test_plateau_error_agrees_with_tau_error():
    x = ar1(1 << 16, 0.9, np.random.default_rng(4)) + 3.0
    a = st.analyse(x)
    assert a["plateau"]
    assert a["error"] == pytest.approx(a["error_tau"], rel=0.25)
    # the naive error underestimates by sqrt(tau)
    naive = x.std(ddof=1) / np.sqrt(x.size)
    assert a["error"] > 3.0 * naive


def test_uncorrelated_series_plateaus_at_block_one():
    x = np.random.default_rng(5).normal(size=4096)
    p = st.plateau(x)
    assert p["converged"] and p["block_size"] <= 4
