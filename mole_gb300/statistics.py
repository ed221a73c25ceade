"""Error analysis of the device-reduced energy series (time-to-sigma).

The sweep kernels reduce the ensemble's E_L sum of every sweep (or block) on
the device; what reaches the host is one number per sweep, the series the
reference analyses offline in scripts/statfor.rs. This module gives

* tau_corr: the integrated autocorrelation time of statfor.rs:30-54,
  tau = 1 + 2 sum_{i=1}^{min(200, n-1)} rho(i), the sum switched off for good
  at the first negative rho, tau >= 1; sigma = sqrt(var tau / n);
* blocking_curve: the blocking error of statfor.rs:57-81 /
  src/vmc/src/vmc.rs:158-167, sqrt((<B^2> - <B>^2) / (n_b - 1)), at block
  sizes 1, 2, 4, ... (whole blocks only) with the error of each estimate,
  err / sqrt(2 (n_b - 1));
* plateau: the smallest block size whose error estimate no estimate at a
  larger block size exceeds by more than two of that estimate's standard
  errors (the blocking curve has flattened out), and that error.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def tau_corr(series, max_lag: int = 200) -> tuple[float, float, float]:
    """(tau, n_eff, sigma of the mean) of a correlated series."""
    x = np.asarray(series, dtype=np.float64)
    n = x.size
    if n < 3:
        return 1.0, float(n), float("nan")
    d = x - x.mean()
    var = float(np.dot(d, d)) / (n - 1)
    if var == 0.0:
        return 1.0, float(n), 0.0
    tau, on = 1.0, True
    for i in range(1, min(max_lag, n - 1) + 1):
        rho = float(np.dot(d[: n - i], d[i:])) / (var * (n - i))
        if rho < 0.0:
            on = False
        if on:
            tau += 2.0 * rho
    tau = max(tau, 1.0)
    return tau, n / tau, math.sqrt(var * tau / n)


@dataclass
class BlockingCurve:
    sizes: np.ndarray
    errors: np.ndarray
    sigmas: np.ndarray  # standard error of each error estimate


def blocking_curve(series, min_blocks: int = 16) -> BlockingCurve:
    x = np.asarray(series, dtype=np.float64)
    sizes, errs, sigs = [], [], []
    size = 1
    while x.size // size >= min_blocks:
        nb = x.size // size
        m = x[: nb * size].reshape(nb, size).mean(axis=1)
        e = math.sqrt(max(float(np.mean(m * m) - np.mean(m) ** 2), 0.0) / (nb - 1))
        sizes.append(size)
        errs.append(e)
        sigs.append(e / math.sqrt(2.0 * (nb - 1)))
        size *= 2
    return BlockingCurve(np.array(sizes), np.array(errs), np.array(sigs))


def plateau(series, min_blocks: int = 16) -> dict:
    """Error of the mean from the blocking plateau; falls back to the largest
    block size when the curve has not flattened (flagged `converged` False)."""
    c = blocking_curve(series, min_blocks)
    if c.sizes.size == 0:
        return {"error": float("nan"), "block_size": 0, "converged": False}
    for k in range(c.sizes.size):
        later = c.errors[k + 1:]
        if later.size and np.all(later <= c.errors[k] + 2.0 * c.sigmas[k + 1:]):
            return {"error": float(c.errors[k]), "block_size": int(c.sizes[k]), "converged": True}
    return {"error": float(c.errors[-1]), "block_size": int(c.sizes[-1]), "converged": False}


def analyse(series) -> dict:
    """Mean, plateau blocking error and tau_corr of a series."""
    x = np.asarray(series, dtype=np.float64)
    tau, neff, sig = tau_corr(x)
    p = plateau(x)
    return {"mean": float(x.mean()) if x.size else float("nan"), "error": p["error"],
            "block_size": p["block_size"], "plateau": p["converged"], "tau_corr": tau, "n_eff": neff,
            "error_tau": sig, "n": int(x.size)}
