"""The FP64-accurate double-float form (MOLE_PREC_DF64) against the CPU oracle.

Every term is a pair of FP32 numbers (about 48 significant bits) on the FP32
pipe; the bar is the FP64 one:
(a) psi, grad ln psi, lap psi / psi, E_L and O_k at identical positions agree
    with the oracle (and the golden vectors) to 1e-10 relative;
(b) short box and Gaussian VMC runs follow the oracle's trajectories, with the
    same acceptance counts and energy / SR sums to 1e-9;
(c) a walker outside FP32's exponent range makes the launch rerun in native
    FP64 on the device, with the native result.
"""
import numpy as np
import pytest

from golden_systems import golden_systems, load_golden
from mole_gb300 import api
from mole_gb300 import system as S
from oracle import oracle as O
from test_gpu_parity import RTOL, close, systems

pytestmark = pytest.mark.gpu

DF_SYSTEMS = ["He", "H2", "He-kappa-poly", "H2+", "SHO", "H-gauss", "Be", "LiH", "Li-2p", "Z-atom-4e"]


@pytest.mark.parametrize("name", DF_SYSTEMS)
def test_eval_df64_matches_oracle(ctx, name):
    s = systems()[name]
    wf = api.WaveFunction(ctx, s)
    W = 257
    pos = np.random.default_rng(7).normal(size=(W, s.n_elec, 3)) * 1.3
    wk = api.Walkers(wf, W, seed=3)
    wk.set_positions(pos)
    before = ctx.df64_reruns()
    g = wk.evaluate(api.PREC_DF64, want_O=s.n_params <= 8)
    assert ctx.df64_reruns() == before  # the double-float kernel produced these values
    r = O.evaluate(s, pos)
    assert close(g["lnpsi"], r["lnpsi"]) < RTOL
    assert np.all(g["sign"] == r["sign"])
    assert close(g["grad"], r["grad"]) < RTOL
    assert close(g["lap"], r["lap"]) < RTOL
    assert close(g["eloc"], r["eloc"]) < RTOL
    if s.n_params <= 8:
        assert close(g["O"], r["O"]) < RTOL


@pytest.mark.parametrize("name", list(golden_systems().keys()))
def test_df64_matches_golden_vectors(ctx, name):
    g = load_golden()[name]
    s = golden_systems()[name]
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, g["pos"].shape[0])
    wk.set_positions(g["pos"])
    r = wk.evaluate(api.PREC_DF64, want_O=False)
    for k in ("lnpsi", "grad", "lap", "eloc"):
        a, b = np.asarray(r[k]), g[k]
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)) < 1e-10, k


@pytest.mark.parametrize("name,move,step,sr", [("He", 0, 0.5, False), ("H2", 1, 0.4, True), ("H2", 0, 0.7, True),
                                               ("Be", 1, 0.3, False), ("LiH", 0, 0.6, False), ("H2+", 0, 1.0, True),
                                               ("Li-2p", 1, 0.3, False), ("SHO", 1, 0.5, True)])
def test_df64_vmc_trajectory_matches_oracle(ctx, name, move, step, sr):
    s = systems()[name]
    sr = sr and s.n_params <= 2
    wf = api.WaveFunction(ctx, s)
    W, n_eq, n_steps, bs = 70, 5, 20, 5
    wk = api.Walkers(wf, W, seed=1234)
    pos0 = wk.positions()
    samp = api.Sampler(wf, api.MetropolisBox(step) if move == 0 else api.MetropolisGaussian(step), wk,
                       precision=api.PREC_DF64, refresh=7)
    before = ctx.df64_reruns()
    res = samp.run(n_eq, n_steps, bs, sr=sr)
    assert ctx.df64_reruns() == before
    ref = O.vmc_run(s, pos0, move=move, step=step, n_eq=n_eq, n_steps=n_steps, block_size=bs, sr=sr, seed=1234)
    assert close(wk.positions(), ref["pos"], rtol=1e-9) < 1e-9
    m, rm = res.moments, ref["moments"]
    assert m[O.MOM_ACCEPT] == rm[O.MOM_ACCEPT] and m[O.MOM_PROPOSED] == rm[O.MOM_PROPOSED]
    for k in (O.MOM_SUM_E, O.MOM_SUM_E2, O.MOM_SUM_BLOCK2):
        assert close(m[k], rm[k], rtol=1e-9) < 1e-9
    assert close(res.time_blocks, ref["time_blocks"], rtol=1e-9) < 1e-9
    if sr:
        assert close(res.sum_O, ref["sum_O"], rtol=1e-9) < 1e-9
        assert close(res.sum_EO, ref["sum_EO"], rtol=1e-9) < 1e-9
        assert close(res.sum_OO, ref["sum_OO"], rtol=1e-9) < 1e-9


def test_df64_long_run_agrees_with_fp64(ctx):
    """Many sweeps of the H2 SR workload: same decisions as native FP64 (equal
    acceptance counts), energy and SR sums to 1e-9."""
    s = S.h2(1.0, 0.5)
    wf = api.WaveFunction(ctx, s)
    out = {}
    for prec in (api.PREC_FP64, api.PREC_DF64):
        wk = api.Walkers(wf, 4096, seed=99)
        out[prec] = (api.Sampler(wf, api.MetropolisGaussian(0.4), wk, precision=prec).run(50, 400, 50, sr=True),
                     wk.positions())
    a, b = out[api.PREC_FP64][0], out[api.PREC_DF64][0]
    assert a.moments[O.MOM_ACCEPT] == b.moments[O.MOM_ACCEPT]
    assert close(a.moments, b.moments, rtol=1e-9) < 1e-9
    assert close(a.sum_O, b.sum_O, rtol=1e-9) < 1e-9
    assert close(a.sum_EO, b.sum_EO, rtol=1e-9) < 1e-9
    assert close(a.sum_OO, b.sum_OO, rtol=1e-9) < 1e-9
    assert close(out[api.PREC_FP64][1], out[api.PREC_DF64][1], rtol=1e-9) < 1e-9


def test_df64_out_of_range_walker_reruns_in_fp64(ctx):
    """One He electron 200 bohr out: its orbital exp(-1.6875 * 200) is below
    FP32's range, so the double-float launch is rerun in native FP64 and the
    results are those of a native FP64 run."""
    s = systems()["He"]
    wf = api.WaveFunction(ctx, s)
    W = 64
    pos = np.random.default_rng(3).normal(size=(W, 2, 3))
    pos[5, 1] = [200.0, 0.0, 0.0]
    res = {}
    for prec in (api.PREC_FP64, api.PREC_DF64):
        wk = api.Walkers(wf, W, seed=5)
        wk.set_positions(pos)
        before = ctx.df64_reruns()
        r = api.Sampler(wf, api.MetropolisBox(0.5), wk, precision=prec).run(0, 10, 5)
        res[prec] = (r.moments, wk.positions(), ctx.df64_reruns() - before)
    assert res[api.PREC_FP64][2] == 0 and res[api.PREC_DF64][2] == 1
    np.testing.assert_array_equal(res[api.PREC_DF64][0], res[api.PREC_FP64][0])
    np.testing.assert_array_equal(res[api.PREC_DF64][1], res[api.PREC_FP64][1])
    wk = api.Walkers(wf, W, seed=5)
    wk.set_positions(pos)
    before = ctx.df64_reruns()
    g = wk.evaluate(api.PREC_DF64, want_O=False)
    assert ctx.df64_reruns() == before + 1
    r = O.evaluate(s, pos, want_O=False)
    assert close(g["eloc"], r["eloc"]) < RTOL


@pytest.mark.parametrize("name,tau", [("He", 0.02), ("Be", 0.005), ("H2", 0.01)])
def test_df64_dmc_trajectory_matches_oracle(ctx, name, tau):
    s = systems()[name]
    wf = api.WaveFunction(ctx, s)
    W = 300
    wk = api.Walkers(wf, W, seed=77)
    pos = wk.positions()
    el = O.evaluate(s, pos, want_O=False)["eloc"]
    dmc = api.DmcRunner(wf, wk, reference_energy=-1.0, precision=api.PREC_DF64)
    before = ctx.df64_reruns()
    e_gpu = dmc.run_block(tau, 6)
    assert ctx.df64_reruns() == before
    e_ref = []
    acc = 0.0
    for t in range(6):
        r = O.dmc_step(s, pos, el, tau=tau, e_ref=-1.0, seed=77, step=t)
        pos, el = r["pos"], r["eloc"]
        e_ref.append(r["energy"])
        acc += r["accepted"]
    assert close(e_gpu, e_ref, rtol=1e-9) < 1e-9
    assert close(wk.positions(), pos, rtol=1e-9) < 1e-9
    assert dmc.accepted == acc


def test_df64_dmc_far_walker_reruns_in_fp64(ctx):
    """A Be walker with an electron 300 bohr out: the double-float DMC steps
    are rerun in native FP64 and give the native result."""
    s = systems()["Be"]
    wf = api.WaveFunction(ctx, s)
    W = 128
    pos = np.random.default_rng(4).normal(size=(W, 4, 3))
    pos[7, 3] = [0.0, 300.0, 0.0]
    out = {}
    for prec in (api.PREC_FP64, api.PREC_DF64):
        wk = api.Walkers(wf, W, seed=8)
        wk.set_positions(pos)
        dmc = api.DmcRunner(wf, wk, reference_energy=-14.6, precision=prec)
        before = ctx.df64_reruns()
        e = dmc.run_block(0.005, 4)
        out[prec] = (np.asarray(e), wk.positions(), ctx.df64_reruns() - before)
    assert out[api.PREC_FP64][2] == 0 and out[api.PREC_DF64][2] == 1
    np.testing.assert_array_equal(out[api.PREC_DF64][0], out[api.PREC_FP64][0])
    np.testing.assert_array_equal(out[api.PREC_DF64][1], out[api.PREC_FP64][1])
