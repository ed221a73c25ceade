"""Stochastic reconfiguration with the neural Jastrow's 9,094 parameters:
network O_k against the oracle, the tensor-core S matrix against a numpy
covariance of the same O_k, the FP64 CG solve against numpy, and training."""
import numpy as np
import pytest

from mole_gb300 import api
from mole_gb300 import system as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def lih_nn(std=0.2, seed=5):
    s = S.lih(neural=True, rng=np.random.default_rng(seed))
    w = np.random.default_rng(seed).normal(0.0, std, size=S.NN_P)
    return s.with_params(np.concatenate([s.params()[:-S.NN_P], w]))


def test_network_log_derivatives_match_oracle(ctx):
    s = lih_nn()
    wf = api.WaveFunction(ctx, s)
    W = 48
    pos = np.random.default_rng(3).normal(size=(W, 4, 3)) * 1.3
    wk = api.Walkers(wf, W)
    wk.set_positions(pos)
    g = wk.evaluate(api.PREC_FP64)["O"]
    r = O.evaluate(s, pos)["O"]
    nw = s.n_params - S.NN_P
    # orbital and Pade parameters in FP64, network parameters in FP32 arithmetic
    np.testing.assert_allclose(g[:, :nw], r[:, :nw], rtol=1e-10, atol=1e-10)
    scale = np.maximum(1.0, np.abs(r[:, nw:]))
    assert np.max(np.abs(g[:, nw:] - r[:, nw:]) / scale) < 2e-4


@pytest.mark.parametrize("n_samples", [3, 6])
def test_tensor_core_s_matrix_and_cg_solve(ctx, n_samples):
    # 3 samples: one GEMM launch over the 3 samples' rows at the solve; 6: a
    # launch over 4 samples when the operand buffer fills (storing S), then
    # one over 2 adding to it
    s = lih_nn(std=0.1)
    wf = api.WaveFunction(ctx, s)
    W = 512
    wk = api.Walkers(wf, W, seed=9)
    samp = api.Sampler(wf, api.MetropolisGaussian(0.3), wk, precision=api.PREC_MIXED)
    samp.run(50, 0, 1)
    Os, Es = [], []
    wk.sr_collect_begin()
    for _ in range(n_samples):
        samp.run(0, 5, 5)
        ev = wk.evaluate(api.PREC_MIXED)
        Os.append(ev["O"])
        Es.append(ev["eloc"])
        wk.sr_collect_sample(api.PREC_MIXED)
    eps = 1e-3
    S_gpu = wk.sr_collect_matrix(eps)
    Ob = np.concatenate(Os)
    Eb = np.concatenate(Es)
    m = Ob.mean(axis=0)
    S_ref = (Ob - m).T @ (Ob - m) / Ob.shape[0] + eps * np.eye(Ob.shape[1])
    d = np.sqrt(np.diag(S_ref))
    err = np.abs(S_gpu - S_ref) / (np.outer(d, d) + 1e-7)
    assert np.max(err) < 0.03, np.max(err)  # BF16 operands, FP32 tile sums, FP64 totals
    assert np.allclose(S_gpu, S_gpu.T)
    delta, g, info = wk.sr_collect_solve(eps, 0.05)
    g_ref = 2.0 * ((Eb[:, None] * Ob).mean(axis=0) - Eb.mean() * m)
    np.testing.assert_allclose(g, g_ref, rtol=2e-3, atol=1e-6)
    x_ref = np.linalg.solve(S_gpu, -0.5 * g)
    assert info[3] < 1e-6
    np.testing.assert_allclose(delta, 0.05 * x_ref, rtol=1e-4, atol=1e-7 * np.max(np.abs(x_ref)))


def test_neural_jastrow_training_beats_pade(ctx):
    # The same LiH determinant and Pade e-e Jastrow with and without the network,
    # both optimised by SR from the same start: the trained network lowers the
    # variational energy and the variance of E_L.
    res = {}
    for neural in (False, True):
        s = S.lih(neural=neural, rng=np.random.default_rng(1))
        wf = api.WaveFunction(ctx, s)
        wk = api.Walkers(wf, 4096, seed=17)
        samp = api.Sampler(wf, api.MetropolisGaussian(0.3), wk, precision=api.PREC_MIXED)
        samp.run(300, 0, 1)
        sr = api.StochasticReconfiguration(0.05, 1e-3, samples=4, sample_every=10)
        vmc = api.VmcRunner(samp, sr)
        vmc.run_optimization(25, 120, 20)
        final = samp.run(100, 2000, 100)
        res[neural] = final
    pade, nn = res[False], res[True]
    assert nn.variance < pade.variance
    assert nn.energy < pade.energy + 2 * np.hypot(nn.error, pade.error)
