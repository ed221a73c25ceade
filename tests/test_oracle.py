"""CPU checks of the oracle itself: it is pinned against the reference's own
known answers before anything is compared with it.

* Philox4x32-10 against the Random123 known-answer vectors.
* The zero-variance harmonic-oscillator eigenstate of
  examples/custom_operator.rs:100-139 (E_L == 1.5 to rounding).
* The Slater-Jastrow evaluator against the reference's own trial functions
  (examples/helium_atom_singlet.rs:60-98, examples/dmc.rs:106-128,
  tests/hydrogen_molecular_ion_lcao.rs:66-92, examples/custom_operator.rs:298-316).
* Finite-difference checks of grad ln psi, the Laplacian and O_k.
* The statistical known answers of tests/helium_lcao.rs:89-137 and
  tests/hydrogen_molecular_ion_lcao.rs:100-141, with the reference's tolerances.
* The constant-psi Metropolis mock of src/metropolis/src/metrop.rs:225-268.
"""
import numpy as np
import pytest

from mole_gb300 import system as S
from oracle import oracle as O


def test_philox_known_answers():
    assert list(O.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_proposal_normals_are_gaussian():
    import ctypes as C

    L = O.lib()
    L.orc_normal_pair.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]
    rng = np.random.default_rng(1)
    a = rng.integers(0, 2 ** 32, size=40000, dtype=np.uint64)
    b = rng.integers(0, 2 ** 32, size=40000, dtype=np.uint64)
    z = np.zeros(2, dtype=np.float32)
    out = np.zeros((a.size, 2))
    for i in range(a.size):
        L.orc_normal_pair(int(a[i]), int(b[i]), z.ctypes.data_as(C.POINTER(C.c_float)))
        out[i] = z
    u = ((a >> 8).astype(np.float64) + 0.5) * 2.0 ** -24
    th = ((b >> 30).astype(np.float64) + (((b >> 6) & 0xFFFFFF).astype(np.float64) + 0.5) * 2.0 ** -24) * np.pi / 2
    r = np.sqrt(-2.0 * np.log(u))
    exact = np.stack([r * np.cos(th), r * np.sin(th)], axis=1)
    assert np.max(np.abs(out - exact)) < 2e-5
    x = out.reshape(-1)
    assert abs(x.mean()) < 0.02 and abs(x.var() - 1.0) < 0.02 and abs((x ** 4).mean() - 3.0) < 0.1


def test_sho_zero_variance():
    s = S.sho_gaussian(np.sqrt(2.0), 1.0)
    pos = np.random.default_rng(3).normal(size=(200, 1, 3)) * 1.5
    r = O.evaluate(s, pos)
    assert np.max(np.abs(r["eloc"] - 1.5)) < 1e-13
    for p in pos[:20]:
        assert abs(O.ref_eloc(O.REF_GAUSSIAN, [np.sqrt(2.0)], p, harmonic=True, omega=1.0) - 1.5) < 1e-13
    # the reference's run: box moves L = 1, 1000 steps, block size 1 (custom_operator.rs:330-343)
    run = O.vmc_run(s, O.init_positions(1, 1, 7, kind=1), move=0, step=1.0, n_eq=1, n_steps=999, block_size=1)
    m = run["moments"]
    mean = m[O.MOM_SUM_E] / m[O.MOM_COUNT]
    var = m[O.MOM_SUM_E2] / m[O.MOM_COUNT] - mean * mean
    assert abs(mean - 1.5) < 1e-14
    assert var < 1e-26


@pytest.mark.parametrize("kind,par,system,nuc,z", [
    (O.REF_HELIUM, [1.69], S.helium_product(1.69), None, [2]),
    (O.REF_STO_H, [0.8], S.hydrogen_sto(0.8), None, [1]),
    (O.REF_H2ION, [1.0, 2.5], S.h2_ion_product(1.0, 2.5), [[1.25, 0, 0], [-1.25, 0, 0]], [1, 1]),
])
def test_slater_jastrow_matches_reference_trial_functions(kind, par, system, nuc, z):
    rng = np.random.default_rng(11)
    pos = rng.normal(size=(50, system.n_elec, 3))
    r = O.evaluate(system, pos)
    for w in range(pos.shape[0]):
        v, g, lap, dp = O.ref_wf(kind, par, pos[w])
        assert abs(np.log(abs(v)) - r["lnpsi"][w]) < 1e-12 * max(1, abs(r["lnpsi"][w]))
        np.testing.assert_allclose(g / v, r["grad"][w], rtol=1e-12, atol=1e-12)
        assert abs(lap / v - r["lap"][w]) < 1e-11 * max(1, abs(lap / v))
        el = O.ref_eloc(kind, par, pos[w], nuc_pos=nuc, nuc_z=z)
        assert abs(el - r["eloc"][w]) < 1e-11 * max(1, abs(el))
        if kind in (O.REF_HELIUM, O.REF_STO_H):
            assert abs(dp / v - r["O"][w][0]) < 1e-12 * max(1, abs(dp / v))


def test_gaussian_trial_function_matches_reference():
    s = S.sho_gaussian(1.3, 0.7)
    pos = np.random.default_rng(5).normal(size=(30, 1, 3))
    r = O.evaluate(s, pos)
    for w in range(30):
        v, g, lap, dp = O.ref_wf(O.REF_GAUSSIAN, [1.3], pos[w])
        np.testing.assert_allclose(g / v, r["grad"][w], rtol=1e-12, atol=1e-13)
        assert abs(lap / v - r["lap"][w]) < 1e-12 * max(1, abs(lap / v))
        assert abs(O.ref_eloc(O.REF_GAUSSIAN, [1.3], pos[w], harmonic=True, omega=0.7) - r["eloc"][w]) < 1e-12


def _systems_for_fd():
    rng = np.random.default_rng(0x5EED + 3)
    he = S.helium(1.6875, 0.3)
    kap = S.System(**{**he.__dict__, "ee_kappa": 0.7, "ee_poly": np.array([0.05, -0.01])})
    return [he, S.h2(), kap, S.random_atom(rng), S.random_atom(rng), S.beryllium(), S.lih(neural=False),
            S.lih(neural=True, rng=np.random.default_rng(4))]


@pytest.mark.parametrize("idx", range(8))
def test_finite_differences(idx):
    s = _systems_for_fd()[idx]
    rng = np.random.default_rng(100 + idx)
    pos = rng.normal(size=(3, s.n_elec, 3)) * 1.2
    r = O.evaluate(s, pos)
    h = 1e-4
    for w in range(pos.shape[0]):
        g = np.zeros((s.n_elec, 3))
        lap = 0.0
        l0 = r["lnpsi"][w]
        for e in range(s.n_elec):
            for c in range(3):
                pp, pm = pos[w].copy(), pos[w].copy()
                pp[e, c] += h
                pm[e, c] -= h
                lp = O.evaluate(s, pp[None], want_O=False)["lnpsi"][0]
                lm = O.evaluate(s, pm[None], want_O=False)["lnpsi"][0]
                g[e, c] = (lp - lm) / (2 * h)
                lap += (lp - 2 * l0 + lm) / (h * h)
        np.testing.assert_allclose(r["grad"][w], g, rtol=2e-6, atol=2e-6)
        lap_over_psi = lap + np.sum(g * g)
        assert abs(r["lap"][w] - lap_over_psi) < 2e-4 * max(1.0, abs(lap_over_psi))
        th = s.params()
        picks = list(range(min(th.size, 6))) + ([th.size - 1, th.size - 4546, 500] if s.nn_on else [])
        for k in picks:
            tp, tm = th.copy(), th.copy()
            hk = 1e-5 * max(1.0, abs(th[k]))
            tp[k] += hk
            tm[k] -= hk
            lp = O.evaluate(s, pos[w][None], theta=tp, want_O=False)["lnpsi"][0]
            lm = O.evaluate(s, pos[w][None], theta=tm, want_O=False)["lnpsi"][0]
            fd = (lp - lm) / (2 * hk)
            assert abs(r["O"][w][k] - fd) < 1e-6 * max(1.0, abs(fd)), (k, r["O"][w][k], fd)


def test_constant_psi_always_accepts():
    # WaveFunctionMock with a constant value: MetropolisBox always accepts (metrop.rs:259-268)
    s = S.System(nuc_pos=[[0, 0, 0]], nuc_z=[0], n_up=1, n_dn=0, basis_center=[0], basis_kind=[S.GTO_1S],
                 basis_exp=[0], exponents=[0.0], coef_up=[[1.0]], coef_dn=np.zeros((0, 1)), pot_kind=S.POT_HARMONIC,
                 omega=1.0)
    run = O.vmc_run(s, O.init_positions(8, 1, 3), move=0, step=1.0, n_eq=0, n_steps=50, block_size=10)
    assert run["moments"][O.MOM_ACCEPT] == run["moments"][O.MOM_PROPOSED] == 400


def test_helium_known_answer():
    # tests/helium_lcao.rs:89-137: alpha = 1.69, MetropolisDiffuse tau = 0.1, 1000 steps, block 100;
    # E(alpha) = alpha^2 - 27 alpha / 8 for the product of 1s functions
    alpha = 1.69
    s = S.helium_product(alpha)
    run = O.vmc_run(s, O.init_positions(16, 2, 21, kind=1), move=2, step=0.1, n_eq=100, n_steps=900, block_size=100,
                    seed=5)
    m = run["moments"]
    mean = m[O.MOM_SUM_E] / m[O.MOM_COUNT]
    std = np.sqrt(m[O.MOM_SUM_E2] / m[O.MOM_COUNT] - mean ** 2)
    exact = alpha * alpha - 27.0 * alpha / 8.0
    assert abs(mean - exact) < 2.0 * std
    err = np.sqrt((m[O.MOM_SUM_BLOCK2] / m[O.MOM_NBLOCKS] - mean ** 2) / (m[O.MOM_NBLOCKS] - 1))
    assert abs(mean - exact) < 5.0 * err


def test_h2_ion_known_answer():
    # tests/hydrogen_molecular_ion_lcao.rs:100-141: MetropolisBox L = 1, |E + 0.565| < std(E_L)
    s = S.h2_ion_product(1.0, 2.5)
    run = O.vmc_run(s, O.init_positions(16, 1, 9, kind=1), move=0, step=1.0, n_eq=100, n_steps=2000, block_size=100,
                    seed=3)
    m = run["moments"]
    mean = m[O.MOM_SUM_E] / m[O.MOM_COUNT]
    std = np.sqrt(m[O.MOM_SUM_E2] / m[O.MOM_COUNT] - mean ** 2)
    assert abs(mean + 0.565) < std


def test_hydrogen_dmc_reaches_exact_energy():
    # examples/dmc.rs:94-149: H atom with an STO guide exp(-0.8 r) (the
    # example's alternative ansatz); DMC projects to the exact -0.5 Ha
    s = S.hydrogen_sto(0.8)
    W = 400
    pos = O.init_positions(W, 1, 17)
    el = O.evaluate(s, pos, want_O=False)["eloc"]
    es = []
    for t in range(600):
        r = O.dmc_step(s, pos, el, tau=0.02, e_ref=-0.5, seed=11, step=t)
        pos, el = r["pos"], r["eloc"]
        if t >= 200:
            es.append(r["energy"])
    assert abs(np.mean(es) + 0.5) < 0.01
