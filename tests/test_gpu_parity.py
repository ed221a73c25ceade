"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

(a) psi, grad ln psi, lap psi / psi, E_L and O_k at identical positions agree
    with the oracle to 1e-10 relative (absolute floor 1e-10) in FP64.
(b) Because the GPU and the oracle consume the same Philox streams, short
    VMC and DMC runs follow the same trajectories: final positions, energy
    sums, acceptance counts and SR sums agree to 1e-9.
"""
import numpy as np
import pytest

from mole_gb300 import api
from mole_gb300 import system as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def close(a, b, rtol=RTOL, floor=1.0):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)
    return np.max(np.abs(a - b) / scale) if a.size else 0.0


def systems():
    rng = np.random.default_rng(0x5EED + 3)
    he = S.helium(1.6875, 0.3)
    kap = S.System(**{**he.__dict__, "ee_kappa": 0.7, "ee_poly": np.array([0.05, -0.01])})
    li = S.System(nuc_pos=[[0, 0, 0]], nuc_z=[3], n_up=2, n_dn=1, basis_center=[0, 0, 0],
                  basis_kind=[S.STO_1S, S.STO_2S, S.STO_2PX], basis_exp=[0, 1, 2], exponents=[2.7, 0.65, 0.6],
                  coef_up=[[1, 0, 0], [0, 1, 0.2]], coef_dn=[[1, 0, 0]], ee_on=True, ee_b=0.8, en_on=True, en_a=1.1,
                  en_coef=[-0.3])
    return {"He": he, "H2": S.h2(), "He-kappa-poly": kap, "H2+": S.h2_ion_product(1.0, 2.5),
            "SHO": S.sho_gaussian(1.3, 0.9), "H-gauss": S.hydrogen_gaussian(1.0), "Be": S.beryllium(),
            "LiH": S.lih(neural=False), "Li-2p": li, "Z-atom-4e": S.random_atom(rng, n_range=(4, 4)),
            "LiH-nn": S.lih(neural=True, rng=np.random.default_rng(21)),
            "Be-nn": _scaled_nn(S.beryllium(neural=True, rng=np.random.default_rng(22)), 0.2)}


def _scaled_nn(s, std):
    """Network weights of a given spread, so the networks' terms are not negligible."""
    w = np.random.default_rng(5).normal(0.0, std, size=s.nn_weights.size)
    return s.with_params(np.concatenate([s.params()[:-w.size], w]))


@pytest.mark.parametrize("name", list(systems().keys()))
def test_eval_matches_oracle_fp64(ctx, name):
    s = systems()[name]
    wf = api.WaveFunction(ctx, s)
    W = 257
    pos = np.random.default_rng(7).normal(size=(W, s.n_elec, 3)) * 1.3
    wk = api.Walkers(wf, W, seed=3)
    wk.set_positions(pos)
    g = wk.evaluate(api.PREC_FP64, want_O=s.n_params <= 8)
    r = O.evaluate(s, pos)
    assert close(g["lnpsi"], r["lnpsi"]) < RTOL
    assert np.all(g["sign"] == r["sign"])
    assert close(g["grad"], r["grad"]) < RTOL
    assert close(g["lap"], r["lap"]) < RTOL
    assert close(g["eloc"], r["eloc"]) < RTOL
    if s.n_params <= 8:
        assert close(g["O"], r["O"]) < RTOL
    np.testing.assert_array_equal(wk.positions(), pos)


@pytest.mark.parametrize("name", ["He", "H2", "Be", "LiH", "Li-2p", "LiH-nn", "Be-nn"])
def test_eval_mixed_precision_close(ctx, name):
    s = systems()[name]
    wf = api.WaveFunction(ctx, s)
    W = 256
    pos = np.random.default_rng(9).normal(size=(W, s.n_elec, 3)) * 1.3
    wk = api.Walkers(wf, W)
    wk.set_positions(pos)
    g = wk.evaluate(api.PREC_MIXED, want_O=s.n_params <= 8)
    r = O.evaluate(s, pos)
    # FP32 orbitals/Jastrow with FP64 contraction and assembly
    assert close(g["eloc"], r["eloc"], floor=1.0) < 2e-4
    assert close(g["grad"], r["grad"], floor=1.0) < 2e-4


@pytest.mark.parametrize("name,move,step", [("He", 0, 0.5), ("H2", 1, 0.4), ("He", 2, 0.1), ("Be", 1, 0.3),
                                            ("Be", 2, 0.05), ("LiH", 0, 0.6), ("H2+", 0, 1.0), ("Li-2p", 2, 0.08),
                                            ("LiH-nn", 1, 0.3), ("Be-nn", 2, 0.05)])
def test_vmc_trajectory_matches_oracle(ctx, name, move, step):
    s = systems()[name]
    wf = api.WaveFunction(ctx, s)
    W, n_eq, n_steps, bs = 70, 5, 20, 5
    wk = api.Walkers(wf, W, seed=1234)
    pos0 = wk.positions()
    np.testing.assert_allclose(pos0, O.init_positions(W, s.n_elec, 1234), rtol=1e-14, atol=1e-14)
    sr = s.n_params <= 8
    samp = api.Sampler(wf, api.MetropolisBox(step) if move == 0 else
                       (api.MetropolisGaussian(step) if move == 1 else api.MetropolisDiffuse(step)), wk, refresh=7)
    res = samp.run(n_eq, n_steps, bs, sr=sr)
    ref = O.vmc_run(s, pos0, move=move, step=step, n_eq=n_eq, n_steps=n_steps, block_size=bs, sr=sr, seed=1234)
    assert close(wk.positions(), ref["pos"], rtol=1e-9) < 1e-9
    m, rm = res.moments, ref["moments"]
    assert m[O.MOM_ACCEPT] == rm[O.MOM_ACCEPT] and m[O.MOM_PROPOSED] == rm[O.MOM_PROPOSED]
    assert m[O.MOM_COUNT] == rm[O.MOM_COUNT] and m[O.MOM_NBLOCKS] == rm[O.MOM_NBLOCKS]
    for k in (O.MOM_SUM_E, O.MOM_SUM_E2, O.MOM_SUM_BLOCK2):
        assert close(m[k], rm[k], rtol=1e-9) < 1e-9
    assert close(res.time_blocks, ref["time_blocks"], rtol=1e-9) < 1e-9
    if sr:
        assert close(res.sum_O, ref["sum_O"], rtol=1e-9) < 1e-9
        assert close(res.sum_EO, ref["sum_EO"], rtol=1e-9) < 1e-9
        assert close(res.sum_OO, ref["sum_OO"], rtol=1e-9) < 1e-9
    assert wk.step == n_eq + n_steps


@pytest.mark.parametrize("name,tau", [("He", 0.02), ("Be", 0.005), ("H2", 0.01)])
def test_dmc_trajectory_matches_oracle(ctx, name, tau):
    s = systems()[name]
    wf = api.WaveFunction(ctx, s)
    W = 300
    wk = api.Walkers(wf, W, seed=77)
    pos = wk.positions()
    el = O.evaluate(s, pos, want_O=False)["eloc"]
    dmc = api.DmcRunner(wf, wk, reference_energy=-1.0)
    e_gpu = dmc.run_block(tau, 6)
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


def test_checkpoint_round_trip(ctx, tmp_path):
    s = S.h2()
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, 100, seed=5)
    api.Sampler(wf, api.MetropolisGaussian(0.4), wk).run(2, 4, 2)
    p = str(tmp_path / "w.ckpt")
    wk.save(p)
    pos, step = wk.positions(), wk.step
    wf2 = api.WaveFunction(ctx, S.h2(alpha=0.9, b=0.1))
    wk2 = api.Walkers(wf2, 100, seed=1)
    wk2.load(p)
    np.testing.assert_array_equal(wk2.positions(), pos)
    assert wk2.step == step
    np.testing.assert_array_equal(wf2.parameters(), s.params())
    with open(p, "r+b") as f:
        f.truncate(60)
    with pytest.raises(api.MoleError) as e:
        wk2.load(p)
    assert e.value.kind == "IoError"


def test_errors_map_to_reference_variants(ctx):
    wf = api.WaveFunction(ctx, S.h2())
    wk = api.Walkers(wf, 16)
    with pytest.raises(api.MoleError) as e:
        api.Sampler(wf, api.MetropolisBox(0.5), wk).run(0, 10, 3)
    assert e.value.kind == "ShapeError"
    with pytest.raises(api.MoleError) as e:
        wf.set_parameters(np.zeros(5))
    assert e.value.kind == "ShapeError"
    bad = wk.positions()
    bad[3, 0, 0] = np.nan
    wk.set_positions(bad)
    with pytest.raises(api.MoleError) as e:
        api.Sampler(wf, api.MetropolisBox(0.5), wk).run(0, 4, 2)
    assert e.value.kind == "FuncError"
