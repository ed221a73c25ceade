"""Golden vectors: the oracle against closed forms of the reference's trial functions.

tests/golden/trial_functions.npz holds ln psi, grad ln psi, lap psi / psi and
E_L of the reference's example/test trial functions at seeded positions,
computed from their closed forms by tests/golden/make_golden.py (numpy,
independent of the oracle's C code). The oracle must reproduce them to 1e-11.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from golden_systems import GOLDEN, golden_systems, load_golden
from oracle import oracle as O

RTOL = 1e-11


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))


@pytest.mark.parametrize("name", list(golden_systems().keys()))
def test_oracle_matches_golden_vectors(name):
    g = load_golden()[name]
    r = O.evaluate(golden_systems()[name], g["pos"], want_O=False)
    assert rel(r["lnpsi"], g["lnpsi"]) < RTOL
    assert rel(r["grad"], g["grad"]) < RTOL
    assert rel(r["lap"], g["lap"]) < RTOL
    assert rel(r["eloc"], g["eloc"]) < RTOL
    assert np.all(r["sign"] == 1.0)


def test_golden_fixture_matches_its_generator(tmp_path):
    here = os.path.dirname(GOLDEN)
    sys.path.insert(0, here)
    try:
        import make_golden
    finally:
        sys.path.remove(here)
    fresh = make_golden.generate()
    z = np.load(GOLDEN)
    assert sorted(fresh) == sorted(z.files)
    for k in z.files:
        np.testing.assert_array_equal(fresh[k], z[k])


def test_zero_variance_golden_point():
    """examples/custom_operator.rs:100-139: the exact harmonic eigenstate (a = sqrt 2, omega = 1) has E_L = 1.5."""
    here = os.path.dirname(GOLDEN)
    sys.path.insert(0, here)
    try:
        import make_golden
    finally:
        sys.path.remove(here)
    pos = np.random.default_rng(3).normal(size=(50, 1, 3)) * 2.0
    _, _, _, el = make_golden.sho(pos, np.sqrt(2.0), 1.0)
    assert np.max(np.abs(el - 1.5)) < 1e-13
