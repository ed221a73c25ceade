"""User observables on the GPU ensemble (Sampler.sample_observables)."""
import numpy as np
import pytest

from mole_gb300 import api
from mole_gb300 import operators as ops
from mole_gb300 import system as S

pytestmark = pytest.mark.gpu


def test_virial_theorem_and_local_energy_consistency(ctx):
    """He product at its optimal exponent 27/16: <V> = -2 <T> (virial theorem),
    <T> = alpha^2, and kinetic + potentials reproduce the device's E_L."""
    a = 27.0 / 16.0
    s = S.helium_product(a)
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, 8192, seed=9)
    samp = api.Sampler(wf, api.MetropolisGaussian(0.5), wk)
    samp.run(200, 0, 1)
    obs = {"T": ops.KineticEnergy(), "V_ion": ops.IonicPotential(s.nuc_pos, s.nuc_z),
           "V_ee": ops.ElectronicPotential(), "H": ops.ElectronicHamiltonian.from_system(s),
           "E_L": type("EL", (ops.LocalOperator,), {"act_on": lambda self, b: b.eloc})()}
    r = samp.sample_observables(obs, 60, every=5, block_size=6)
    T, V = r.mean["T"], r.mean["V_ion"] + r.mean["V_ee"]
    assert abs(r.mean["H"] - r.mean["E_L"]) < 1e-9
    assert abs(T - a * a) < 5 * r.error["T"] + 1e-3
    assert abs(V + 2 * T) < 5 * np.hypot(r.error["V_ion"] + r.error["V_ee"], 2 * r.error["T"]) + 2e-3


def test_custom_harmonic_operator(ctx):
    """examples/custom_operator.rs: the harmonic Hamiltonian as a user operator
    on the exact eigenstate -- every sample is 1.5."""
    s = S.sho_gaussian(np.sqrt(2.0), 1.0)
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, 1024, seed=3)
    samp = api.Sampler(wf, api.MetropolisBox(1.0), wk)
    r = samp.sample_observables({"H": ops.HarmonicHamiltonian(1.0)}, 10, every=3)
    assert abs(r.mean["H"] - 1.5) < 1e-12
