"""Local operators on walker batches evaluated by the CPU oracle.

The built-in operators of mole_gb300.operators restate the reference's
(src/operator/src/operator.rs, src/vmc/src/operators.rs): kinetic + ionic +
electronic potential must equal the local energy, and the harmonic
Hamiltonian of examples/custom_operator.rs gives E_L = 1.5 on its exact
eigenstate (zero variance, examples/custom_operator.rs:100-139)."""
import numpy as np

from mole_gb300 import operators as ops
from mole_gb300 import system as S
from oracle import oracle as O


def batch(system, pos):
    r = O.evaluate(system, pos)
    return ops.WalkerBatch(pos, r["lnpsi"], r["sign"], r["grad"], r["lap"], r["eloc"], r["O"])


def test_hamiltonian_terms_sum_to_the_local_energy():
    for s in (S.h2(), S.beryllium(cusp=True), S.lih(neural=False)):
        pos = np.random.default_rng(1).normal(size=(40, s.n_elec, 3)) * 1.2
        b = batch(s, pos)
        h = ops.ElectronicHamiltonian.from_system(s).act_on(b)
        np.testing.assert_allclose(h, b.eloc, rtol=1e-12, atol=1e-12)


def test_harmonic_hamiltonian_on_the_exact_eigenstate():
    s = S.sho_gaussian(np.sqrt(2.0), 1.0)
    pos = np.random.default_rng(2).normal(size=(100, 1, 3)) * 2.0
    e = ops.HarmonicHamiltonian(1.0).act_on(batch(s, pos))
    assert np.max(np.abs(e - 1.5)) < 1e-13


def test_wavefunction_value_and_parameter_gradient():
    s = S.helium_product(1.69)
    pos = np.random.default_rng(3).normal(size=(20, 2, 3))
    b = batch(s, pos)
    psi = ops.WavefunctionValue().act_on(b)
    r = np.linalg.norm(pos, axis=-1).sum(axis=1)
    np.testing.assert_allclose(psi, np.exp(-1.69 * r), rtol=1e-12)
    np.testing.assert_allclose(ops.ParameterGradient().act_on(b)[:, 0], -r, rtol=1e-12)
