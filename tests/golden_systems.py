"""The systems of tests/golden/trial_functions.npz as descriptors of this
package (the fixture's generator defines them by their closed forms)."""
import numpy as np

from mole_gb300 import system as S

GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "trial_functions.npz")


def golden_systems() -> dict:
    return {
        "H-sto": S.hydrogen_sto(0.8),
        "He-product": S.helium_product(1.69),
        "He-pade": S.helium(1.6875, 0.3),
        "H2+product": S.h2_ion_product(1.0, 2.5),
        "SHO": S.sho_gaussian(1.3, 0.9),
        "H2-pade": S.h2(1.0, 0.5, 0.7),
    }


def load_golden() -> dict:
    z = np.load(GOLDEN)
    out = {}
    for key in z.files:
        name, field = key.split("/")
        out.setdefault(name, {})[field] = z[key]
    return out
