"""Edge sizes through the C ABI against the oracle: one walker, walker counts
around a warp and a CTA (partial tiles), equilibration-only runs, a batch of
one system with one walker, and rejected empty or inconsistent inputs."""
import numpy as np
import pytest

from mole_gb300 import api
from mole_gb300 import system as S
from mole_gb300._lib import STATUS
from oracle import oracle as O


def _lib_kind(rc):
    return STATUS.get(rc, "OK" if rc == 0 else "Unknown")

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))


@pytest.mark.parametrize("W", [1, 31, 63, 65, 129])
def test_vmc_trajectories_at_odd_walker_counts(ctx, W):
    s = S.beryllium(cusp=True)
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, W, seed=W)
    pos0 = wk.positions()
    r = api.Sampler(wf, api.MetropolisGaussian(0.3), wk).run(2, 4, 2)
    ref = O.vmc_run(s, pos0, move=1, step=0.3, n_eq=2, n_steps=4, block_size=2, seed=W)
    assert rel(wk.positions(), ref["pos"]) < 1e-9
    assert r.moments[O.MOM_ACCEPT] == ref["moments"][O.MOM_ACCEPT]
    assert rel(r.moments[O.MOM_SUM_E], ref["moments"][O.MOM_SUM_E]) < 1e-9


def test_equilibration_only_run(ctx):
    s = S.h2()
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, 100, seed=2)
    pos0 = wk.positions()
    r = api.Sampler(wf, api.MetropolisGaussian(0.4), wk).run(5, 0, 1)
    ref = O.vmc_run(s, pos0, move=1, step=0.4, n_eq=5, n_steps=0, block_size=1, seed=2)
    assert r.moments[O.MOM_COUNT] == 0 and r.time_blocks.size == 0
    assert rel(wk.positions(), ref["pos"]) < 1e-9
    assert wk.step == 5


def test_single_walker_evaluation(ctx):
    s = S.lih(neural=False)
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, 1)
    pos = np.random.default_rng(1).normal(size=(1, 4, 3))
    wk.set_positions(pos)
    g = wk.evaluate(api.PREC_FP64)
    r = O.evaluate(s, pos)
    assert rel(g["eloc"], r["eloc"]) < 1e-10 and rel(g["grad"], r["grad"]) < 1e-10


def test_batch_of_one_system_one_walker(ctx):
    s = S.random_atom(np.random.default_rng(4), n_range=(7, 7))
    b = api.Batch(ctx, [s], [1], seeds=[9], widths=[0.25])
    pos0 = b.positions(0)
    r = b.run(api.MetropolisGaussian(1.0), 3, 4, 2, precision=api.PREC_FP64)[0]
    ref = O.vmc_run(s, pos0, move=1, step=0.25, n_eq=3, n_steps=4, block_size=2, seed=9)
    assert rel(b.positions(0), ref["pos"]) < 1e-9
    assert r.moments[O.MOM_ACCEPT] == ref["moments"][O.MOM_ACCEPT]


def test_rejected_inputs(ctx):
    wf = api.WaveFunction(ctx, S.h2())
    with pytest.raises(api.MoleError) as e:
        api.Walkers(wf, 0)
    assert e.value.kind == "ShapeError"
    wk = api.Walkers(wf, 8)
    bad = np.zeros(7 * 2 * 3)
    rc = wf.lib.mole_walkers_set_positions(wk.h, api.dptr(bad), bad.size)
    assert _lib_kind(rc) == "ShapeError"
    with pytest.raises(api.MoleError) as e:
        api.Batch(ctx, [], [])
    assert e.value.kind == "ShapeError"
    with pytest.raises(api.MoleError) as e:
        api.Batch(ctx, [S.h2()], [0])
    assert e.value.kind == "ShapeError"
