"""CPU checks of the reference arithmetic restated in oracle/compat.py and of
the host-side logic the GPU path uses instead (statistics, SR, comb)."""
import numpy as np

from mole_gb300 import api
from oracle import compat


def test_reversed_division_stores_reciprocal_gradient():
    psi = np.array([0.5, 2.0])
    dpsi = np.array([[0.25, 4.0], [1.0, -2.0]])
    np.testing.assert_allclose(compat.stored_parameter_gradient(psi, dpsi), 1.0 / dpsi)


def test_reference_sr_matrix_centring_differs_from_covariance():
    rng = np.random.default_rng(1)
    O = rng.normal(1.0, 0.3, size=(500, 3))
    psi = np.ones(500)
    S_ref = compat.construct_sr_matrix(O, psi)
    ob = O.mean(axis=0)
    cov = (O.T @ O) / 500 - np.outer(ob, ob)
    expected = (O.T @ O) / 500 - ob.sum() ** 2
    expected[np.diag_indices(3)] *= 1.01
    np.testing.assert_allclose(S_ref, expected, rtol=1e-12)
    assert np.max(np.abs(S_ref - cov)) > 1.0


def test_physics_sr_matches_device_reduction_formula():
    rng = np.random.default_rng(2)
    O = rng.normal(size=(1000, 2))
    E = -1.1 + 0.3 * O[:, 0] + rng.normal(size=1000) * 0.1
    d_ref = compat.physics_sr_update(0.05, 1e-3, O, E)
    r = api.MonteCarloResult(energy=E.mean(), error=0.0, variance=0.0, acceptance=0.5,
                             moments=np.array([1000, E.sum(), (E * E).sum(), 0, 0, 0, 0]), time_blocks=np.zeros(0),
                             sum_O=O.sum(0), sum_EO=(E[:, None] * O).sum(0), sum_OO=O.T @ O)
    g = r.energy_gradient()
    ob = O.mean(0)
    S = (O.T @ O) / 1000 - np.outer(ob, ob) + 1e-3 * np.eye(2)
    np.testing.assert_allclose(0.05 * np.linalg.solve(S, -0.5 * g), d_ref, rtol=1e-10)


def test_blocking_error_formula_matches_reference():
    rng = np.random.default_rng(3)
    x = rng.normal(size=(4, 200)).cumsum(axis=1) * 0.01 + rng.normal(size=(4, 200))
    bs = 20
    flat = x.reshape(-1)
    ref = compat.blocking_error(flat, bs)
    bm = x.reshape(4, -1, bs).mean(axis=2)
    mom = np.array([flat.size, flat.sum(), (flat ** 2).sum(), (bm ** 2).sum(), bm.size, 0, 1])
    assert abs(api.blocking_error(mom) - ref) < 1e-12


def test_comb_is_unbiased_and_low_variance():
    rng = np.random.default_rng(4)
    w = rng.exponential(size=1000)
    counts = np.bincount(compat.comb(w, 0.37), minlength=1000)
    expect = w * 1000 / w.sum()
    assert counts.sum() == 1000
    assert np.all(np.abs(counts - expect) < 1.0 + 1e-12)
    parents, mw = compat.sr_brancher(w, rng)
    assert parents.size == 1000 and abs(mw - w.mean()) < 1e-15
