"""Walkers split across ranks (one GPU each): the exchange step of VMC + SR.

Walkers are independent Markov chains, so ranks share nothing while they
sweep. The one exchange is per SR iteration, where the reference's
VmcRunner concatenates its workers' samples before the optimizer step
(src/vmc/src/vmc.rs:78-89, concatenate_worker_data at 108-130): here every
rank's device-reduced sums (moments, time blocks, sum O_k, sum E O_k,
sum O_k O_l) are summed with one all_reduce of a flat FP64 vector, so every
rank computes the same parameter update from the ensemble of all ranks.
"""
from __future__ import annotations

import numpy as np


def _dist():
    import torch.distributed as dist

    return dist


def world() -> tuple[int, int]:
    """(rank, world size); (0, 1) when torch.distributed is not initialised."""
    dist = _dist()
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(), dist.get_world_size()


def allreduce_sum(values: np.ndarray, group=None) -> np.ndarray:
    """Sum a flat FP64 array over the ranks of `group` (identity with one rank)."""
    import torch

    dist = _dist()
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return np.asarray(values, dtype=np.float64).copy()
    t = torch.from_numpy(np.ascontiguousarray(values, dtype=np.float64).copy())
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def allreduce_result(result, group=None):
    """A MonteCarloResult whose sums cover the walkers of every rank; energy,
    blocking error, variance and acceptance are re-derived from them."""
    from .api import MonteCarloResult, blocking_error

    parts = [result.moments, result.time_blocks]
    sr = result.sum_O is not None
    if sr:
        parts += [result.sum_O, result.sum_EO, np.ravel(result.sum_OO)]
    sizes = [np.size(p) for p in parts]
    flat = allreduce_sum(np.concatenate([np.ravel(p) for p in parts]), group)
    out, o = [], 0
    for n in sizes:
        out.append(flat[o:o + n])
        o += n
    mom = out[0]
    n = mom[0]
    E = mom[1] / n if n else float("nan")
    var = mom[2] / n - E * E if n else float("nan")
    kw = {}
    if sr:
        P = result.sum_O.size
        kw = dict(sum_O=out[2], sum_EO=out[3], sum_OO=out[4].reshape(P, P))
    return MonteCarloResult(E, blocking_error(mom), var, mom[5] / max(mom[6], 1.0), mom, out[1], **kw)
