"""The team kernel's named-barrier protocol (mole_gb300/csrc/team.cuh), run
as a model on the CPU.

Each warp of a team is a generator of the barrier operations and
shared-memory accesses its code performs, in program order: bar.sync and
bar.arrive with their ids and thread counts, writes of a move's slot and
reads that expect a given move's value. A scheduler interleaves the warps as
the hardware may (random and greedy orders), with named-barrier semantics:
a barrier completes when its count of threads has arrived, every arrival of
one generation names the same count, and a warp in bar.sync waits until the
completion. The model checks that no schedule deadlocks, that no barrier is
left with arrivals at exit and that every read sees the write of the move it
expects. Two planted faults (two exchange slots instead of four; a missing
arrival) must be caught, which shows that the model can fail."""
import random

import pytest

SNAP_READ, SNAP_WRITTEN, START = 5, 3, 7


def team_warps(total, n_eq, n_elec, slots=4, arrive=True):
    """The operation streams of the team's warps for `total` sweeps, as the
    kernel issues them (move m = it * n_elec + e; barrier id 1 + e)."""
    n_steps = total - n_eq
    moves = total * n_elec
    snap_n = 128 if n_elec == 2 else 64

    def move_count(m):
        return 96 if m + 1 < moves else 64

    def one_body(e):
        if n_elec == 2 and moves > 0:
            yield ("w", "xn", e % slots, e)
            yield ("arrive", START, 64) if e == 0 else ("arrive", 1, 96)
        for it in range(total):
            m = it * n_elec + e
            if n_elec == 2:
                yield ("w", "ratio", m % slots, m)
                yield ("sync", 1 + e, move_count(m))
                yield ("r", "dj", m % slots, m)
            if it + 1 < total and n_elec == 2:
                yield ("w", "xn", (m + 2) % slots, m + 2)
                if arrive:
                    yield ("arrive", 2 - e, 96)
            if it < n_eq:
                continue
            k = it - n_eq
            if k >= 2:
                yield ("sync", SNAP_READ + (k & 1), snap_n)
            yield ("w", "snap%d" % e, k & 1, k)
            yield ("arrive", SNAP_WRITTEN + (k & 1), snap_n)
        for k in range(max(n_steps - 2, 0), n_steps):
            yield ("sync", SNAP_READ + (k & 1), snap_n)

    def pair():
        if n_elec != 2:
            return
        if moves > 0:
            yield ("sync", START, 64)
        for it in range(total):
            for e in range(2):
                m = it * 2 + e
                yield ("r", "xn", m % slots, m)
                yield ("w", "dj", m % slots, m)
                yield ("sync", 1 + e, move_count(m))
                yield ("r", "ratio", m % slots, m)
            if it < n_eq:
                continue
            k = it - n_eq
            if k >= 2:
                yield ("sync", SNAP_READ + (k & 1), snap_n)
            yield ("w", "snapP", k & 1, k)
            yield ("arrive", SNAP_WRITTEN + (k & 1), snap_n)
        for k in range(max(n_steps - 2, 0), n_steps):
            yield ("sync", SNAP_READ + (k & 1), snap_n)

    def local_energy():
        for k in range(n_steps):
            yield ("sync", SNAP_WRITTEN + (k & 1), snap_n)
            yield ("r", "snap0", k & 1, k)
            if n_elec == 2:
                yield ("r", "snap1", k & 1, k)
                yield ("r", "snapP", k & 1, k)
            yield ("arrive", SNAP_READ + (k & 1), snap_n)

    warps = {"one_body_0": one_body(0), "pair": pair(), "local_energy": local_energy()}
    if n_elec == 2:
        warps["one_body_1"] = one_body(1)
    return warps


def run_schedule(warps, rng, priority=None):
    """Interleaves the warps; returns None or a description of the fault."""
    op = {k: next(g, None) for k, g in warps.items()}
    waiting = {}
    barriers = {}
    memory = {}
    while True:
        ready = [k for k in op if op[k] is not None and k not in waiting]
        if not ready:
            if waiting or any(v is not None for v in op.values()):
                return "deadlock: %s" % sorted(waiting.items())
            left = {i: b[0] for i, b in barriers.items() if b[0]}
            return "arrivals left at exit: %s" % left if left else None
        if priority is not None and rng.random() < 0.8:
            k = min(ready, key=priority.index)
        else:
            k = rng.choice(ready)
        o = op[k]
        if o[0] in ("sync", "arrive"):
            _, bid, n = o
            b = barriers.setdefault(bid, [0, None, []])
            if b[0] == 0:
                b[1] = n
            elif b[1] != n:
                return "barrier %d: counts %d and %d in one generation" % (bid, b[1], n)
            b[0] += 32
            if o[0] == "sync":
                b[2].append(k)
                waiting[k] = bid
            if b[0] > n:
                return "barrier %d: more than %d threads" % (bid, n)
            if b[0] == n:
                for w in b[2]:
                    del waiting[w]
                barriers[bid] = [0, None, []]
        elif o[0] == "w":
            memory[(o[1], o[2])] = o[3]
        else:
            seen = memory.get((o[1], o[2]))
            if seen != o[3]:
                return "%s read %s slot %d: move %s, expected %d" % (k, o[1], o[2], seen, o[3])
        op[k] = next(warps[k], None)


def faults(n_runs, seed, **kw):
    rng = random.Random(seed)
    found = []
    for i in range(n_runs):
        n_elec = 2 if i % 4 else 1
        total = rng.randint(1, 8)
        n_eq = rng.randint(0, total - 1)
        warps = team_warps(total, n_eq, n_elec, **kw)
        priority = None if i % 3 == 0 else rng.sample(sorted(warps), len(warps))
        f = run_schedule(warps, rng, priority)
        if f:
            found.append((total, n_eq, n_elec, f))
    return found


def test_team_protocol_has_no_deadlock_or_race():
    assert faults(1500, 1) == []


def test_team_protocol_edge_sizes():
    rng = random.Random(5)
    for n_elec in (1, 2):
        for total, n_eq in ((1, 0), (2, 0), (2, 1), (3, 0), (3, 2), (0, 0)):
            for _ in range(20):
                assert run_schedule(team_warps(total, n_eq, n_elec), rng) is None


@pytest.mark.parametrize("planted,expect", [
    (dict(slots=2), "read"),
    (dict(arrive=False), "deadlock"),
])
def test_team_protocol_model_catches_planted_faults(planted, expect):
    found = faults(600, 2, **planted)
    assert found and any(expect in f[3] for f in found)
