"""CPU checks of the C ABI library: it loads without a GPU and exports every
function include/mole_gpu.h declares (no compute calls are made)."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "mole_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mole_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("mole_ctx_create", "mole_system_create", "mole_walkers_create", "mole_eval", "mole_vmc_run",
              "mole_sr_update", "mole_dmc_run", "mole_checkpoint_save", "mole_last_error_string"):
        assert n in names


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="CUDA toolkit absent")
def test_library_exports_every_declared_symbol():
    from mole_gb300 import _lib, build

    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.SIGNATURES) == set(declared_functions())
    assert lib.mole_abi_version() == 1
