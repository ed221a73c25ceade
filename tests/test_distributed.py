"""Two gloo ranks on the CPU: the SR iteration's exchange of device-reduced sums.

Each rank holds its own walkers' sums; after allreduce_result both ranks see
the sums of the whole ensemble and derive the same energy, blocking error,
acceptance and energy gradient, hence the same parameter update.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_result(rank):
    from mole_gb300.api import MonteCarloResult

    rng = np.random.default_rng(100 + rank)
    P = 3
    mom = np.array([1000.0, -1130.0 + rank, 1300.0 + 2 * rank, 12.0 + rank, 10.0, 600.0 + rank, 900.0])
    O = rng.normal(size=P)
    OO = np.outer(O, O) + np.eye(P)
    return MonteCarloResult(0.0, 0.0, 0.0, 0.0, mom, rng.normal(size=4), O * 10, O * -11, OO * 1000)


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from mole_gb300.distributed import allreduce_result

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r = allreduce_result(_rank_result(rank))
        out.put((rank, r.moments, r.time_blocks, r.sum_O, r.sum_EO, r.sum_OO, r.energy, r.error, r.acceptance,
                 r.energy_gradient()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_see_the_ensemble_sums():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict((v[0], v[1:]) for v in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, b = _rank_result(0), _rank_result(1)
    mom = a.moments + b.moments
    for rank in (0, 1):
        m, tb, sO, sEO, sOO, E, err, acc, g = got[rank]
        np.testing.assert_allclose(m, mom)
        np.testing.assert_allclose(tb, a.time_blocks + b.time_blocks)
        np.testing.assert_allclose(sO, a.sum_O + b.sum_O)
        np.testing.assert_allclose(sOO, a.sum_OO + b.sum_OO)
        assert E == pytest.approx(mom[1] / mom[0])
        assert acc == pytest.approx(mom[5] / mom[6])
    # both ranks take the same step
    np.testing.assert_array_equal(got[0][-1], got[1][-1])
    assert got[0][6] == got[1][6]


def test_single_process_is_identity():
    from mole_gb300.distributed import allreduce_result, world

    assert world() == (0, 1)
    r = _rank_result(0)
    s = allreduce_result(r)
    np.testing.assert_array_equal(s.moments, r.moments)
    np.testing.assert_array_equal(s.sum_OO, r.sum_OO)
