"""The CUDA path (FP64, through the C ABI) against the golden vectors of the
reference's trial functions (tests/golden/trial_functions.npz) to 1e-10."""
import numpy as np
import pytest

from golden_systems import golden_systems, load_golden
from mole_gb300 import api

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(golden_systems().keys()))
def test_gpu_matches_golden_vectors(ctx, name):
    g = load_golden()[name]
    s = golden_systems()[name]
    wf = api.WaveFunction(ctx, s)
    wk = api.Walkers(wf, g["pos"].shape[0])
    wk.set_positions(g["pos"])
    r = wk.evaluate(api.PREC_FP64, want_O=False)
    for k in ("lnpsi", "grad", "lap", "eloc"):
        a, b = np.asarray(r[k]), g[k]
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)) < 1e-10, k
