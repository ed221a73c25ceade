"""The reference's own known-answer tests, run on the GPU path through the
host mirror (their structure follows the reference's tests), plus the
statistical parity checks (b): energies within 2 sigma by blocking analysis,
mixed precision against FP64, SR optimisation and DMC projections."""
import numpy as np
import pytest

from mole_gb300 import api
from mole_gb300 import system as S

pytestmark = pytest.mark.gpu


def test_custom_operator_zero_variance(ctx):
    # examples/custom_operator.rs:100-139: exact eigenstate a = sqrt(2 / omega),
    # MetropolisBox(1.0), Runner.run(1000, 1); |E - 1.5| < 1e-15 and std < 1e-15
    wf = api.WaveFunction(ctx, S.sho_gaussian(np.sqrt(2.0), 1.0))
    wk = api.Walkers(wf, 4096, init=api.INIT_UNIFORM)
    r = api.Runner(api.Sampler(wf, api.MetropolisBox(1.0), wk)).run(1000, 1)
    assert abs(r.energy - 1.5) < 1e-14
    assert r.variance < 1e-26


def test_helium_lcao(ctx):
    # tests/helium_lcao.rs:89-138: alpha = 1/(1/1.69), MetropolisDiffuse(0.1), run(1000, 100)
    alpha = 1.0 / (1.0 / 1.69)
    wf = api.WaveFunction(ctx, S.helium_product(alpha))
    wk = api.Walkers(wf, 2048, init=api.INIT_UNIFORM)
    r = api.Runner(api.Sampler(wf, api.MetropolisDiffuse(0.1), wk)).run(1000, 100)
    exact = alpha * alpha - 27.0 * alpha / 8.0
    assert abs(r.energy - exact) < 2.0 * np.sqrt(r.variance)
    assert abs(r.energy - exact) < 4.0 * r.error


def test_hydrogen_molecular_ion_lcao(ctx):
    # tests/hydrogen_molecular_ion_lcao.rs:100-142: MetropolisBox(1.0), run(10000, 100), |E + 0.565| < std
    wf = api.WaveFunction(ctx, S.h2_ion_product(1.0, 2.5))
    wk = api.Walkers(wf, 1024, init=api.INIT_UNIFORM)
    r = api.Runner(api.Sampler(wf, api.MetropolisBox(1.0), wk)).run(10000, 100)
    assert abs(r.energy + 0.565) < np.sqrt(r.variance)
    assert 0.0 < r.acceptance < 1.0


def test_sho_optimize(ctx):
    # tests/sho_optimize.rs:117-141 with the corrected gradient: optimise the Gaussian
    # exponent from a = 1 (zeta = 1) down to the exact eigenstate energy 1.5
    wf = api.WaveFunction(ctx, S.sho_gaussian(1.0, 1.0))
    wk = api.Walkers(wf, 1024)
    vmc = api.VmcRunner(api.Sampler(wf, api.MetropolisDiffuse(0.1), wk), api.StochasticReconfiguration(0.5, 1e-3))
    _, energies, errors, _ = vmc.run_optimization(20, 200, 10)
    assert abs(energies[-1] - 1.5) < max(errors[-1], 1e-3)
    assert abs(wf.parameters()[0] - 0.5) < 0.02


def test_steepest_descent_moves_downhill(ctx):
    wf = api.WaveFunction(ctx, S.sho_gaussian(1.0, 1.0))
    wk = api.Walkers(wf, 2048)
    vmc = api.VmcRunner(api.Sampler(wf, api.MetropolisDiffuse(0.1), wk), api.SteepestDescent(0.2))
    _, energies, _, _ = vmc.run_optimization(10, 100, 10)
    assert energies[-1] < energies[0] - 0.1


class _Grad:
    def __init__(self, g):
        self.g = np.asarray(g, dtype=np.float64)

    def energy_gradient(self):
        return self.g.copy()


@pytest.mark.parametrize("name", ["momentum", "nesterov", "lbfgs"])
def test_host_optimizers_through_vmc_runner(ctx, name):
    """MomentumDescent, NesterovMomentum and OnlineLbfgs (optimizers.rs:45-192)
    driving VmcRunner on the harmonic well: every update the runner applies is
    the optimizer's rule on the device-reduced gradient (a fresh optimizer fed
    the recorded gradients reproduces the parameter trajectory), the momentum
    forms lower the energy from psi's exponent 1 (E = 1.875) toward 1/2
    (E = 1.5), and the reference's online L-BFGS (1e-10 first step, duplicated
    curvature pairs) stays finite at a small step."""
    make = {"momentum": lambda: api.MomentumDescent(0.05, 0.5, 1),
            "nesterov": lambda: api.NesterovMomentum(0.05, 0.5, 1),
            "lbfgs": lambda: api.OnlineLbfgs(0.02, 2, 1)}[name]
    wf = api.WaveFunction(ctx, S.sho_gaussian(1.0, 1.0))
    wk = api.Walkers(wf, 4096, seed=5)
    p0 = wf.parameters().copy()
    rec = []
    vmc = api.VmcRunner(api.Sampler(wf, api.MetropolisDiffuse(0.1), wk), make())
    _, energies, _, _ = vmc.run_optimization(
        12, 100, 10, callback=lambda it, r, w: rec.append((r.energy_gradient(), w.parameters().copy())))
    opt, p = make(), p0
    for g, p_after in rec:
        p = p + opt.compute_parameter_update(p, _Grad(g))
        np.testing.assert_allclose(p, p_after, rtol=1e-12, atol=1e-15)
    assert np.all(np.isfinite(energies))
    if name != "lbfgs":
        assert energies[-1] < energies[0] - 0.05


def test_vmc_energy_statistics_fp64_vs_mixed(ctx):
    # helium singlet (alpha 1.6875, beta 0.3): the mixed form agrees with FP64 within 2 sigma
    res = {}
    for prec in (api.PREC_FP64, api.PREC_MIXED):
        wf = api.WaveFunction(ctx, S.helium(1.6875, 0.3))
        wk = api.Walkers(wf, 4096, seed=11)
        res[prec] = api.Sampler(wf, api.MetropolisBox(0.5), wk, precision=prec).run(500, 2000, 100)
    a, b = res[api.PREC_FP64], res[api.PREC_MIXED]
    assert abs(a.energy - b.energy) < 2.0 * np.hypot(a.error, b.error)
    assert abs(a.acceptance - b.acceptance) < 0.01
    # He with this Jastrow lies between the Hartree-Fock-like -2.85 and the exact -2.9037
    assert -2.91 < a.energy < -2.85


def test_h2_sr_optimisation_lowers_energy(ctx):
    # the H2 VMC + SR workload at reduced size: alpha = 1.0, b = 0.5, Gaussian moves 0.4, eps 1e-3, step 0.05
    wf = api.WaveFunction(ctx, S.h2(1.0, 0.5))
    wk = api.Walkers(wf, 8192)
    vmc = api.VmcRunner(api.Sampler(wf, api.MetropolisGaussian(0.4), wk), api.StochasticReconfiguration(0.05, 1e-3))
    _, energies, errors, _ = vmc.run_optimization(12, 220, 20)
    assert energies[-1] < energies[0] - 5 * errors[-1]
    assert -1.18 < energies[-1] < -1.05


@pytest.mark.parametrize("name,system,tau,exact,tol", [
    ("H", S.hydrogen_sto(0.8), 0.02, -0.5, 0.01),
    ("He", S.helium(2.0, 0.3), 0.01, -2.9037, 0.015),
])
def test_dmc_projects_to_exact_ground_state(ctx, name, system, tau, exact, tol):
    # DmcRunner::diffuse (src/dmc/src/dmc.rs:69-153) with a nodeless guide: the
    # fixed-node energy is the exact ground-state energy. The guides satisfy
    # the nuclear (and, for He, the e-e) cusp: the reference's weights are
    # not capped, so a guide whose E_L diverges at a coalescence lets the
    # population collapse onto a few walkers.
    wf = api.WaveFunction(ctx, system)
    wk = api.Walkers(wf, 8192, seed=3)
    api.Sampler(wf, api.MetropolisDiffuse(tau), wk).run(200, 0, 1)
    dmc = api.DmcRunner(wf, wk, reference_energy=exact + 0.1)
    energies, errors = dmc.diffuse(tau, 6000, 200, 5)
    assert abs(energies[-1] - exact) < tol, (energies[-1], errors[-1])
    assert 0.9 < dmc.acceptance <= 1.0


def test_be_dmc_with_cusp_guide_and_weight_cutoff_is_stable(ctx):
    """Be DMC with the Pade guide: the e-n term restores the nuclear cusp and
    E_L is clipped to E_ref +- 2/sqrt(tau) in the weight factor only; the
    population energy settles near Be's fixed-node energy instead of
    running away to the walkers that sit on the nucleus."""
    s = S.beryllium(cusp=True)
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, 8192, seed=31)
    api.Sampler(wf, api.MetropolisDiffuse(0.02), wk).run(100, 0, 1)
    tau = 0.005
    dmc = api.DmcRunner(wf, wk, -14.6, precision=api.PREC_MIXED, eloc_cutoff=2.0 / np.sqrt(tau))
    dmc.run_block(tau, 400)
    e = dmc.run_block(tau, 400)
    assert np.all(np.isfinite(e))
    assert -14.70 < float(np.mean(e)) < -14.62
    assert 0.95 < dmc.acceptance <= 1.0
    # walkers the FP32 orbitals put exactly on the |r1| = |r2| node are rare
    assert dmc.node_kills < 1e-4 * 8192 * 800
