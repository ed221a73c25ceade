"""The ragged-batch path (one persistent launch over many systems) against the oracle.

Each system of a batch consumes the Philox streams keyed by its own seed, the
streams the oracle's per-system VMC consumes, so in FP64 every system's
trajectory, acceptance counts and energy sums agree with the oracle's run of
that system alone (to 1e-9). Electron counts 2..10 (spin blocks up to 5 + 5)
with 1s/2s/2p Slater orbitals, Pade e-e and e-n Jastrows are covered, with
walker counts that leave partial tiles.
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


def atoms():
    """One atom for each electron count 2..10, plus a neutral-ish Z=10 ion with 10 electrons."""
    rng = np.random.default_rng(0x5EED + 30)
    out = [S.random_atom(rng, n_range=(n, n)) for n in range(2, 11)]
    out.append(S.random_atom(rng, z_range=(10, 10), n_range=(10, 10)))
    return out


def widths_of(systems):
    return np.array([0.6 / np.sqrt(float(s.nuc_z[0])) for s in systems])


@pytest.mark.parametrize("move,scale", [(api.MetropolisGaussian, 1.0), (api.MetropolisBox, 2.0)])
def test_batch_trajectories_match_oracle(ctx, move, scale):
    systems = atoms()
    W = np.array([37, 64, 70, 5, 129, 33, 96, 41, 65, 50])
    seeds = np.arange(len(systems)) * 7 + 11
    widths = widths_of(systems)
    b = api.Batch(ctx, systems, W, seeds=seeds, widths=widths)
    b.tile = 64
    pos0 = [b.positions(k) for k in range(len(b))]
    for k, s in enumerate(systems):
        np.testing.assert_allclose(pos0[k], O.init_positions(int(W[k]), s.n_elec, int(seeds[k])), rtol=1e-14,
                                   atol=1e-14)
    n_eq, n_steps, bs = 3, 6, 3
    res = b.run(move(scale), n_eq, n_steps, bs, precision=api.PREC_FP64, refresh=4)
    for k, s in enumerate(systems):
        ref = O.vmc_run(s, pos0[k], move=move(1.0).kind, step=float(widths[k] * scale), n_eq=n_eq, n_steps=n_steps,
                        block_size=bs, seed=int(seeds[k]))
        m, rm = res[k].moments, ref["moments"]
        assert close(b.positions(k), ref["pos"]) < 1e-9, s.name
        assert m[O.MOM_ACCEPT] == rm[O.MOM_ACCEPT] and m[O.MOM_PROPOSED] == rm[O.MOM_PROPOSED], s.name
        assert m[O.MOM_COUNT] == rm[O.MOM_COUNT] and m[O.MOM_NBLOCKS] == rm[O.MOM_NBLOCKS]
        for j in (O.MOM_SUM_E, O.MOM_SUM_E2, O.MOM_SUM_BLOCK2):
            assert close(m[j], rm[j]) < 1e-9, (s.name, j)
    assert b.step == n_eq + n_steps


def test_batch_graph_replays_continue_the_streams(ctx):
    systems = atoms()[::3]
    W = np.array([40, 77, 64, 10])
    b = api.Batch(ctx, systems, W, seeds=[1, 2, 3, 4], widths=widths_of(systems))
    pos0 = [b.positions(k) for k in range(len(b))]
    for _ in range(3):
        b.run(api.MetropolisGaussian(1.0), 1, 2, 1, precision=api.PREC_FP64)
    assert b.step == 9 and b.graph_launches == 3
    for k, s in enumerate(systems):
        p = pos0[k]
        for c in range(3):
            p = O.vmc_run(s, p, move=S.MOVE_GAUSS, step=float(widths_of(systems)[k]), n_eq=1, n_steps=2,
                          block_size=1, seed=k + 1, step0=3 * c)["pos"]
        assert close(b.positions(k), p) < 1e-9, s.name


def test_batch_matches_single_system_path(ctx):
    """A 2 + 2 system in a batch follows the fixed-size kernel's trajectory."""
    be = S.beryllium()
    lih = S.lih(neural=False)
    b = api.Batch(ctx, [be, lih], [100, 70], seeds=[5, 6], widths=[0.3, 0.5])
    b.run(api.MetropolisGaussian(1.0), 4, 8, 4, precision=api.PREC_FP64)
    for k, (s, w, sd, st) in enumerate([(be, 100, 5, 0.3), (lih, 70, 6, 0.5)]):
        wf = api.WaveFunction(ctx, s)
        wk = api.Walkers(wf, w, seed=sd)
        r = api.Sampler(wf, api.MetropolisGaussian(st), wk).run(4, 8, 4)
        assert close(wk.positions(), b.positions(k)) < 1e-9


def test_batch_mixed_precision_energies_agree_with_fp64(ctx):
    systems = atoms()[:6]
    W = np.full(len(systems), 2048)
    widths = widths_of(systems)
    out = {}
    for prec in (api.PREC_FP64, api.PREC_MIXED):
        b = api.Batch(ctx, systems, W, seeds=np.arange(6) + 100, widths=widths)
        b.run(api.MetropolisGaussian(1.0), 200, 0, 1, precision=prec)
        out[prec] = b.run(api.MetropolisGaussian(1.0), 0, 400, 20, precision=prec)
    for k in range(len(systems)):
        a, m = out[api.PREC_FP64][k], out[api.PREC_MIXED][k]
        assert np.isfinite(a.energy) and np.isfinite(m.energy)
        assert abs(a.energy - m.energy) < 4.0 * np.hypot(a.error, m.error) + 1e-4 * abs(a.energy), systems[k].name
        assert 0.2 < m.acceptance < 0.95


def test_batch_helium_product_energy(ctx):
    """Jastrow-free He product psi = exp(-alpha (r1 + r2)) inside a ragged batch:
    E = alpha^2 - 27 alpha / 8 (tests/helium_lcao.rs:89-137)."""
    alpha = 1.6875
    systems = [S.helium_product(alpha)] + atoms()[4:7]
    b = api.Batch(ctx, systems, [8192, 300, 500, 700], widths=[0.5, 0.3, 0.3, 0.3])
    b.run(api.MetropolisGaussian(1.0), 200, 0, 1)
    r = b.run(api.MetropolisGaussian(1.0), 0, 400, 20)[0]
    exact = alpha * alpha - 27.0 * alpha / 8.0
    assert abs(r.energy - exact) < 4.0 * r.error + 1e-4


def test_batch_autotune_leaves_chains_untouched(ctx, tmp_path, monkeypatch):
    monkeypatch.setenv("MOLE_GB300_TILE_CACHE", str(tmp_path / "tiles.json"))
    systems = atoms()
    W = np.array([300, 200, 500, 100, 400, 256, 129, 64, 700, 90])
    b = api.Batch(ctx, systems, W, widths=widths_of(systems))
    pos0 = [b.positions(k) for k in range(len(b))]
    t = b.autotune(api.MetropolisGaussian(1.0), api.PREC_MIXED, sweeps=4)
    assert not t["cached"] and t["tile"] in t["timings"] and len(t["timings"]) >= 3
    assert all(ms > 0 for ms in t["timings"].values())
    for k in range(len(b)):
        np.testing.assert_array_equal(b.positions(k), pos0[k])
    assert b.step == 0
    t2 = b.autotune(api.MetropolisGaussian(1.0), api.PREC_MIXED, sweeps=4)
    assert t2["cached"] and t2["tile"] == t["tile"]
    # a tuned batch still follows the oracle
    b.tile = 128
    res = b.run(api.MetropolisGaussian(1.0), 1, 2, 2, precision=api.PREC_FP64)
    for k in (0, 8):
        ref = O.vmc_run(systems[k], pos0[k], move=S.MOVE_GAUSS, step=float(widths_of(systems)[k]), n_eq=1,
                        n_steps=2, block_size=2, seed=0x5EED + k)
        assert close(b.positions(k), ref["pos"]) < 1e-9
        assert res[k].moments[O.MOM_ACCEPT] == ref["moments"][O.MOM_ACCEPT]


def test_batch_rejections(ctx):
    systems = atoms()[:2]
    b = api.Batch(ctx, systems, [32, 32])
    with pytest.raises(api.MoleError) as e:
        b.run(api.MetropolisDiffuse(0.01), 0, 2, 1)
    assert e.value.kind == "Unsupported"
    with pytest.raises(api.MoleError) as e:
        b.run(api.MetropolisGaussian(1.0), 0, 5, 2)
    assert e.value.kind == "ShapeError"
    with pytest.raises(api.MoleError) as e:
        api.Batch(ctx, [S.lih(neural=True)], [32])
    assert e.value.kind == "Unsupported"
    with pytest.raises(api.MoleError) as e:
        b.tile = 48
    assert e.value.kind == "InvalidArgument"
    # a 5 + 5 system exists for batches but has no single-system kernels
    big = [s for s in atoms() if s.n_elec == 10][0]
    wf = api.WaveFunction(ctx, big)
    wk = api.Walkers(wf, 16)
    with pytest.raises(api.MoleError) as e:
        api.Sampler(wf, api.MetropolisGaussian(0.2), wk).run(0, 2, 1)
    assert e.value.kind == "Unsupported"
    bad = b.positions(1)
    bad[3, 0, 0] = np.nan
    b.set_positions(1, bad)
    with pytest.raises(api.MoleError) as e:
        b.run(api.MetropolisGaussian(1.0), 0, 2, 1)
    assert e.value.kind in ("FuncError", "LinalgError")
