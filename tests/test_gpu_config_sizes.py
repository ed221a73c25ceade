"""Oracle parity at the sizes and launch geometries the bench times.

The other parity tests run tens to hundreds of walkers; these run the
workloads' own ensembles through the same C ABI calls, so the launch shapes
the bench times -- whole waves of SMs x resident CTAs with the walkers split
evenly, the packed FP64 kernel (224-thread CTAs, FP32-screened proposals
whose FP64 evaluation is packed across warps), ~1,000 CTAs of partial sums
reduced in a fixed order, the ragged batch's persistent work queue, the
multi-block comb scan -- are checked against the CPU oracle on the same
random streams:

* He singlet (alpha 1.6875, beta 0.3), box 0.5 bohr: the 1,024 walkers of its
  workload, and 65,536 walkers (the packed kernel's box path);
* H2 Slater-Pade (alpha 1.0, b 0.5), Gaussian 0.4 bohr, SR sums: 65,536
  walkers in native FP64 (packed kernel) and in the double-float form;
* a hydrogen atom (1s STO) at 40,000 walkers with SR sums (the packed
  kernel's one-electron form);
* Be DMC (Pade guide), 131,072 VMC-equilibrated walkers, tau 0.005, comb
  every step;
* the full 256-system ragged batch (583,055 walkers, N = 2..10) in FP64;
* LiH with the pair networks at 16,384 walkers: evaluation against the oracle,
  and one full SR sample's tensor-core S matrix within the bound its BF16
  operands and FP32 tile sums allow.

The bar is the trajectory bar of the smaller tests: positions to 1e-9,
identical acceptance counts, sums to 1e-9.
"""
import numpy as np
import pytest

from mole_gb300 import api
from mole_gb300 import system as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def close(a, b, floor=1.0):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)) if a.size else 0.0


def check_vmc(res, wk, ref, sr):
    assert close(wk.positions(), ref["pos"]) < 1e-9
    m, rm = res.moments, ref["moments"]
    assert m[O.MOM_ACCEPT] == rm[O.MOM_ACCEPT] and m[O.MOM_PROPOSED] == rm[O.MOM_PROPOSED]
    assert m[O.MOM_COUNT] == rm[O.MOM_COUNT] and m[O.MOM_NBLOCKS] == rm[O.MOM_NBLOCKS]
    for k in (O.MOM_SUM_E, O.MOM_SUM_E2, O.MOM_SUM_BLOCK2):
        assert close(m[k], rm[k]) < 1e-9, k
    assert close(res.time_blocks, ref["time_blocks"]) < 1e-9
    if sr:
        for a, b in ((res.sum_O, ref["sum_O"]), (res.sum_EO, ref["sum_EO"]), (res.sum_OO, ref["sum_OO"])):
            assert close(a, b) < 1e-9


def h_atom():
    return S.System(nuc_pos=[[0, 0, 0]], nuc_z=[1], n_up=1, n_dn=0, basis_center=[0], basis_kind=[S.STO_1S],
                    basis_exp=[0], exponents=[0.9], coef_up=[[1.0]], coef_dn=np.zeros((0, 1)), name="H-1s")


@pytest.mark.parametrize("name,W,move,step,prec,sr", [
    ("He", 1024, 0, 0.5, api.PREC_FP64, False),
    ("He", 65536, 0, 0.5, api.PREC_FP64, False),
    ("H2", 65536, 1, 0.4, api.PREC_FP64, True),
    ("H2", 65536, 1, 0.4, api.PREC_DF64, True),
    ("H", 40000, 1, 0.8, api.PREC_FP64, True),
])
def test_vmc_at_workload_size_matches_oracle(ctx, name, W, move, step, prec, sr):
    s = {"He": S.helium(1.6875, 0.3), "H2": S.h2(1.0, 0.5), "H": h_atom()}[name]
    wf = api.WaveFunction(ctx, s)
    seed = 0x5EED + W + move
    wk = api.Walkers(wf, W, seed=seed)
    pos0 = wk.positions()
    n_eq, n_steps, bs = 2, 4, 2
    samp = api.Sampler(wf, api.MetropolisBox(step) if move == 0 else api.MetropolisGaussian(step), wk,
                       precision=prec)
    res = samp.run(n_eq, n_steps, bs, sr=sr)
    ref = O.vmc_run_threads(s, pos0, move=move, step=step, n_eq=n_eq, n_steps=n_steps, block_size=bs, sr=sr,
                            seed=seed)
    check_vmc(res, wk, ref, sr)
    assert res.acceptance > 0.3


def test_be_dmc_at_workload_size_matches_oracle(ctx):
    """From VMC-equilibrated walkers, as the DMC workload starts. (An
    unequilibrated N(0, 1) ensemble of this size holds walkers within ~1e-6
    bohr of a node, where the reference's drift-diffusion rule throws an
    electron hundreds of bohr and rounding at 1e-16 decides the outcome; one
    such walker's weight then takes over the comb.)"""
    s = S.beryllium()
    wf = api.WaveFunction(ctx, s)
    W, tau = 131072, 0.005
    wk = api.Walkers(wf, W, seed=0x5EED + 5)
    api.Sampler(wf, api.MetropolisGaussian(0.3), wk).run(200, 0, 1)
    pos = wk.positions()
    t0 = wk.step  # the DMC steps continue the walkers' random-stream position
    el = O.evaluate(s, pos, want_O=False)["eloc"]
    dmc = api.DmcRunner(wf, wk, reference_energy=-14.6)
    e_gpu = dmc.run_block(tau, 2)
    e_ref, acc = [], 0.0
    for t in range(2):
        r = O.dmc_step(s, pos, el, tau=tau, e_ref=-14.6, seed=0x5EED + 5, step=t0 + t)
        pos, el = r["pos"], r["eloc"]
        e_ref.append(r["energy"])
        acc += r["accepted"]
    assert close(e_gpu, e_ref) < 1e-9
    assert close(wk.positions(), pos) < 1e-9
    assert dmc.accepted == acc


def test_full_ragged_batch_matches_oracle(ctx):
    from concurrent.futures import ThreadPoolExecutor

    systems, walkers, widths = api.ragged_batch(256)
    assert int(walkers.sum()) == 583055
    seeds = np.arange(len(systems), dtype=np.int64) * 13 + 5
    b = api.Batch(ctx, systems, walkers, seeds=seeds, widths=widths)
    pos0 = [b.positions(k) for k in range(len(b))]
    n_eq, n_steps, bs = 1, 2, 1
    res = b.run(api.MetropolisGaussian(1.0), n_eq, n_steps, bs, precision=api.PREC_FP64)

    def one(k):
        return O.vmc_run(systems[k], pos0[k], move=1, step=float(widths[k]), n_eq=n_eq, n_steps=n_steps,
                         block_size=bs, seed=int(seeds[k]))

    with ThreadPoolExecutor(max_workers=O.hardware_threads()) as ex:
        refs = list(ex.map(one, range(len(systems))))
    for k, ref in enumerate(refs):
        m, rm = res[k].moments, ref["moments"]
        assert close(b.positions(k), ref["pos"]) < 1e-9, systems[k].name
        assert m[O.MOM_ACCEPT] == rm[O.MOM_ACCEPT] and m[O.MOM_PROPOSED] == rm[O.MOM_PROPOSED], systems[k].name
        for j in (O.MOM_SUM_E, O.MOM_SUM_E2, O.MOM_SUM_BLOCK2):
            assert close(m[j], rm[j]) < 1e-9, (systems[k].name, j)


def lih_nn(std=0.1, seed=5):
    s = S.lih(neural=True, rng=np.random.default_rng(seed))
    w = np.random.default_rng(seed).normal(0.0, std, size=S.NN_P)
    return s.with_params(np.concatenate([s.params()[:-S.NN_P], w]))


def test_lih_neural_evaluation_at_workload_size(ctx):
    """LiH with the pair networks, 16,384 walkers (its workload's ensemble):
    ln psi, sign, grad ln psi, lap psi / psi and E_L of the FP64 form against
    the oracle at 1e-10, and the network O_k of the first 1,024 walkers within
    the network bar of the smaller test (FP32 backward pass, 2e-4)."""
    s = lih_nn(std=0.2)
    wf = api.WaveFunction(ctx, s)
    W = 16384
    wk = api.Walkers(wf, W, seed=0x5EED + 4)
    api.Sampler(wf, api.MetropolisGaussian(0.3), wk, precision=api.PREC_MIXED).run(50, 0, 1)
    pos = wk.positions()
    g = wk.evaluate(api.PREC_FP64, want_O=False)
    r = O.evaluate(s, pos, want_O=False)
    for k in ("lnpsi", "grad", "lap", "eloc"):
        assert close(g[k], r[k]) < 1e-10, k
    assert np.all(g["sign"] == r["sign"])
    sub = api.Walkers(wf, 1024, seed=1)
    sub.set_positions(pos[:1024])
    go = sub.evaluate(api.PREC_FP64)["O"]
    ro = O.evaluate(s, pos[:1024])["O"]
    nw = s.n_params - S.NN_P
    np.testing.assert_allclose(go[:, :nw], ro[:, :nw], rtol=1e-10, atol=1e-10)
    assert np.max(np.abs(go[:, nw:] - ro[:, nw:]) / np.maximum(1.0, np.abs(ro[:, nw:]))) < 2e-4


def test_s_matrix_of_one_full_sample_within_bf16_bound(ctx):
    """One SR sample of the LiH neural workload (16,384 walkers, 9,094
    parameters): the tcgen05 S matrix against float64 numpy on the O_k the
    evaluation returns. The GEMM's operands are a = bf16(O - c), c the mean
    O_k of the sample's first 1,024 walkers (unit roundoff 2^-8, so a product
    carries at most 2^-7 relative error), summed in FP32 inside a tile over
    the sample's K = 16,384 walkers (at most K 2^-24 of the sum of
    magnitudes), so |S_gpu - S_ref|_ij <= (2^-7 + K 2^-24) B_ij with
    B_ij = sum_k |a_ki| |a_kj| / K, plus the FP32 rounding of c's own sums;
    checked on 320 rows (the orbital/Pade parameters, both networks' first
    and last layers) against every column."""
    s = lih_nn(std=0.1)
    wf = api.WaveFunction(ctx, s)
    W = 16384
    wk = api.Walkers(wf, W, seed=9)
    api.Sampler(wf, api.MetropolisGaussian(0.3), wk, precision=api.PREC_MIXED).run(50, 0, 1)
    ev = wk.evaluate(api.PREC_MIXED)
    wk.sr_collect_begin()
    wk.sr_collect_sample(api.PREC_MIXED)
    eps = 1e-3
    S_gpu = wk.sr_collect_matrix(eps)
    Ob = ev["O"]
    A = Ob - Ob.mean(axis=0)
    Ac = Ob - Ob[:1024].mean(axis=0)  # the operand the GEMM sees, before rounding
    P = Ob.shape[1]
    rng = np.random.default_rng(0)
    rows = np.unique(np.concatenate([np.arange(8), np.arange(P - 64, P), rng.choice(P, 248, replace=False)]))
    S_ref = A[:, rows].T @ A / W
    S_ref[np.arange(rows.size), rows] += eps
    B = np.abs(Ac[:, rows]).T @ np.abs(Ac) / W
    bound = (2.0 ** -7 + W * 2.0 ** -24) * B + 1e-12
    err = np.abs(S_gpu[rows] - S_ref)
    assert np.all(err <= bound), float(np.max(err / bound))
    assert np.allclose(S_gpu, S_gpu.T)
