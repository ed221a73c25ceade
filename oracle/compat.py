"""Reference ("compat") arithmetic on per-sample lists, in numpy.

TEST INFRASTRUCTURE ONLY. This restates, bug for bug, the host-side
arithmetic the reference applies to its stored samples, so that tests can
show exactly where the GPU path's corrected ("physics") arithmetic departs
from it:

* Vector / Scalar divides the other way round (src/operator/src/traits.rs:149-150),
  so a stored "Parameter gradient" sample is psi / (psi * dpsi/dp) = 1/(dpsi/dp)
  (src/vmc/src/operators.rs:14-18 with src/montecarlo/src/samplers.rs:89-90).
* compute_energy_gradient (src/optimize/src/util.rs:6-46).
* construct_sr_matrix subtracts sum_ij <O_i><O_j> from EVERY element and then
  scales the diagonal by 1 + 1e-2 (src/optimize/src/optimizers.rs:191-234).
* the blocking error of src/vmc/src/vmc.rs:133-172 over chunks(block_size).
* SRBrancher (src/dmc/src/branching.rs:7-40): N multinomial draws with
  probabilities proportional to u32(w * N / w_max), new weights = mean weight.
"""
from __future__ import annotations

import numpy as np


def stored_parameter_gradient(psi: np.ndarray, dpsi: np.ndarray) -> np.ndarray:
    """Per-sample "Parameter gradient" as the reference stores it."""
    psi = np.asarray(psi, dtype=np.float64)[:, None]
    act_on = np.asarray(dpsi, dtype=np.float64) * psi  # Vector(dpsi) * Scalar(psi)
    return psi / act_on  # Vector / Scalar, reversed


def energy_gradient(wf_values, par_grads, energies, energy_mean) -> np.ndarray:
    """util.rs:36-46: mean_n 2 (psi_i / psi)_n (E_n - E)."""
    wf = np.asarray(wf_values, dtype=np.float64)[:, None]
    pg = np.asarray(par_grads, dtype=np.float64)
    el = np.asarray(energies, dtype=np.float64)[:, None]
    return np.mean(2.0 * (pg / wf) * (el - energy_mean), axis=0)


def construct_sr_matrix(par_grads, wf_values) -> np.ndarray:
    """optimizers.rs:191-234, including the centring and diagonal scaling it applies."""
    pg = np.asarray(par_grads, dtype=np.float64)
    wf = np.asarray(wf_values, dtype=np.float64)[:, None]
    o = pg / wf
    n, p = o.shape
    s = np.zeros((p, p))
    for k in range(n):
        s += np.outer(o[k], o[k]) / n
    oavg = o.mean(axis=0)
    for i in range(p):
        for j in range(p):
            s -= oavg[i] * oavg[j]  # subtracted from every element
    s[np.diag_indices(p)] *= 1.0 + 1e-2
    return s


def sr_update(step_size, par_grads, wf_values, energies, energy_mean) -> np.ndarray:
    """StochasticReconfiguration::compute_parameter_update (optimizers.rs:237-252)."""
    g = energy_gradient(wf_values, par_grads, energies, energy_mean)
    s = construct_sr_matrix(par_grads, wf_values)
    return step_size * np.linalg.solve(s, -0.5 * g)


def physics_sr_update(step_size, eps, O, E) -> np.ndarray:
    """The corrected update the GPU path implements, from per-sample
    O_k = d ln psi / d p_k and E_L: S = cov(O) + eps I, g = 2 cov(E, O)."""
    O = np.asarray(O, dtype=np.float64)
    E = np.asarray(E, dtype=np.float64)
    ob = O.mean(axis=0)
    S = (O.T @ O) / O.shape[0] - np.outer(ob, ob) + eps * np.eye(O.shape[1])
    g = 2.0 * ((E[:, None] * O).mean(axis=0) - E.mean() * ob)
    return step_size * np.linalg.solve(S, -0.5 * g)


def running_mean(x) -> float:
    """VmcRunner::mean (vmc.rs:174-179): a += (b - a) / (n + 1)."""
    a = 0.0
    for n, b in enumerate(x):
        a = a + (b - a) / (n + 1)
    return a


def blocking_error(samples, block_size: int) -> float:
    """vmc.rs:157-169: blocks are consecutive chunks of block_size samples."""
    s = np.asarray(samples, dtype=np.float64)
    mean = running_mean(s)
    chunks = [s[i:i + block_size] for i in range(0, s.size, block_size)]
    bm = np.array([running_mean(c) for c in chunks])
    b2 = running_mean(bm * bm)
    return float(np.sqrt((b2 - mean * mean) / (len(chunks) - 1)))


def sr_brancher(weights, rng: np.random.Generator) -> tuple[np.ndarray, float]:
    """branching.rs:15-39: parents drawn N times with probability proportional
    to the u32-truncated normalised weights; every new weight is the mean."""
    w = np.asarray(weights, dtype=np.float64)
    n = w.size
    mean_w = w.sum() / n
    iw = np.floor(w * (n / w.max())).astype(np.uint64).astype(np.float64)
    parents = rng.choice(n, size=n, p=iw / iw.sum())
    return parents, mean_w


def comb(weights, u: float) -> np.ndarray:
    """Systematic resampling with one uniform: parent of new walker k is the
    first j with cumsum(w)[j] > (k + u) * sum(w) / N."""
    w = np.asarray(weights, dtype=np.float64)
    c = np.cumsum(w)
    t = (np.arange(w.size) + u) * (c[-1] / w.size)
    return np.minimum(np.searchsorted(c, t, side="right"), w.size - 1)


def statfor_correlation(data, max_steps: int = 200):
    """scripts/statfor.rs:30-54: tau = 1 + 2 sum_i rho(i), i = 1..min(200, n-1),
    the sum switched off for good at the first negative rho; tau >= 1;
    returns (tau, n / tau, sqrt(var tau / n)) with var of ddof 1 (statfor.rs:23-26)."""
    x = np.asarray(data, dtype=np.float64)
    n = x.size
    mean = x.mean()
    var = np.sum((mean - x) ** 2) / (n - 1)
    tau, f = 1.0, 1.0
    for i in range(1, min(max_steps, n - 1) + 1):
        corr = np.sum((x[: n - i] - mean) * (x[i:] - mean)) / (var * (n - i))
        if corr < 0.0:
            f = 0.0
        tau += 2.0 * corr * f
    tau = max(tau, 1.0)
    return tau, n / tau, float(np.sqrt(var * tau / n))


def statfor_blocking(data, min_left: int = 20, n_sizes: int = 100):
    """scripts/statfor.rs:57-81: for block sizes 1..n/20 (step max(1, (n/20)/100))
    the error sqrt((<B^2> - <B>^2) / (n / size - 1)) over data.chunks(size),
    the last chunk possibly partial. Returns [(size, error)]."""
    x = np.asarray(data, dtype=np.float64)
    n = x.size
    large = n // min_left
    step = max(large // n_sizes, 1)
    out = []
    for size in range(1, large + 1, step):
        nblocks = n // size
        means = np.array([c.mean() for c in np.array_split(x, range(size, n, size))])
        ave_sq = np.mean(means ** 2)
        ave = np.mean(means)
        out.append((size, float(np.sqrt((ave_sq - ave * ave) / (nblocks - 1)))))
    return out
