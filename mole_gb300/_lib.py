"""ctypes binding of libmole_gpu.so (the C ABI of include/mole_gpu.h).

The library is built in-tree by mole_gb300.build; loading fails loudly when
it is missing or CUDA is unavailable -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib: C.CDLL | None = None

OK = 0
STATUS = {
    1: "LinalgError", 2: "ShapeError", 3: "FuncError", 4: "OperatorValueAccessError", 5: "DataAccessError",
    6: "EmptyCacheError", 100: "CudaError", 101: "InvalidArgument", 102: "Timeout", 103: "Unsupported", 104: "IoError",
}
NMOM = 7


class MoleError(RuntimeError):
    """Raised for a non-zero mole_status; .code holds the status, .kind the
    errors::Error variant name of the reference (src/errors/src/lib.rs:8-15)."""

    def __init__(self, code: int, msg: str):
        self.code = code
        self.kind = STATUS.get(code, "Unknown")
        super().__init__(f"{self.kind} ({code}): {msg}")


class SystemDesc(C.Structure):
    _fields_ = [
        ("n_nuclei", C.c_int32), ("nuc_pos", C.POINTER(C.c_double)), ("nuc_charge", C.POINTER(C.c_int32)),
        ("n_up", C.c_int32), ("n_dn", C.c_int32), ("n_basis", C.c_int32),
        ("basis_center", C.POINTER(C.c_int32)), ("basis_kind", C.POINTER(C.c_int32)),
        ("basis_exp", C.POINTER(C.c_int32)), ("n_exp", C.c_int32),
        ("coef_up", C.POINTER(C.c_double)), ("coef_dn", C.POINTER(C.c_double)),
        ("ee_on", C.c_int32), ("ee_npoly", C.c_int32), ("ee_kappa", C.c_double), ("cusp_anti", C.c_double),
        ("cusp_para", C.c_double), ("en_on", C.c_int32), ("en_coef", C.POINTER(C.c_double)),
        ("nn_on", C.c_int32), ("pot_kind", C.c_int32), ("omega", C.c_double),
    ]


class VmcOpts(C.Structure):
    _fields_ = [("move", C.c_int32), ("step", C.c_double), ("n_eq", C.c_int32), ("n_steps", C.c_int32),
                ("block_size", C.c_int32), ("sr", C.c_int32), ("precision", C.c_int32), ("refresh", C.c_int32)]


class DmcOpts(C.Structure):
    _fields_ = [("tau", C.c_double), ("e_ref", C.c_double), ("n_steps", C.c_int32), ("precision", C.c_int32),
                ("refresh", C.c_int32), ("eloc_cutoff", C.c_double)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol declared in include/mole_gpu.h
SIGNATURES = {
    "mole_abi_version": (C.c_int32, []),
    "mole_last_error_string": (C.c_char_p, []),
    "mole_ctx_create": (C.c_int, [C.c_int32, C.POINTER(_P)]),
    "mole_ctx_destroy": (C.c_int, [_P]),
    "mole_ctx_set_stream": (C.c_int, [_P, _P]),
    "mole_sync": (C.c_int, [_P]),
    "mole_ctx_enable_timing": (C.c_int, [_P, C.c_int32]),
    "mole_ctx_kernel_time": (C.c_int, [_P, C.c_int32, _D, C.POINTER(C.c_int64)]),
    "mole_probe_peaks": (C.c_int, [_P, _D, _D]),
    "mole_ctx_df64_reruns": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "mole_math_check": (C.c_int, [_P, C.c_int32, _D, C.c_int64, _D]),
    "mole_ctx_device_info": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "mole_system_create": (C.c_int, [_P, C.POINTER(SystemDesc), _D, C.c_int32, C.POINTER(_P)]),
    "mole_system_destroy": (C.c_int, [_P]),
    "mole_num_params": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "mole_params_get": (C.c_int, [_P, _D, C.c_int32]),
    "mole_params_set": (C.c_int, [_P, _D, C.c_int32]),
    "mole_num_electrons": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "mole_walkers_create": (C.c_int, [_P, C.c_int32, C.c_uint64, C.POINTER(_P)]),
    "mole_walkers_destroy": (C.c_int, [_P]),
    "mole_walkers_count": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "mole_walkers_init": (C.c_int, [_P, C.c_int32, C.c_double]),
    "mole_walkers_set_positions": (C.c_int, [_P, _D, C.c_int64]),
    "mole_walkers_get_positions": (C.c_int, [_P, _D, C.c_int64]),
    "mole_walkers_get_step": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "mole_walkers_set_step": (C.c_int, [_P, C.c_uint64]),
    "mole_eval": (C.c_int, [_P, C.c_int32, _D, _D, _D, _D, _D, _D]),
    "mole_vmc_run": (C.c_int, [_P, C.POINTER(VmcOpts), _D, _D, _D, _D, _D]),
    "mole_vmc_run_noalloc": (C.c_int, [_P, C.c_void_p, C.c_int32, C.c_uint64, C.c_uint64, C.POINTER(VmcOpts),
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mole_sr_update": (C.c_int, [_P, C.c_int32, C.c_double, _D, _D, _D, _D, C.c_double, C.c_double, _D, _D]),
    "mole_sr_collect_begin": (C.c_int, [_P]),
    "mole_sr_collect_sample": (C.c_int, [_P, C.c_int32]),
    "mole_sr_collect_solve": (C.c_int, [_P, C.c_double, C.c_double, C.c_int32, C.c_double, _D, _D, _D]),
    "mole_sr_collect_matrix": (C.c_int, [_P, C.c_double, _D]),
    "mole_dmc_run": (C.c_int, [_P, C.POINTER(DmcOpts), _D, _D]),
    "mole_dmc_node_kills": (C.c_int, [_P, _D]),
    "mole_batch_create": (C.c_int, [_P, C.c_int32, C.POINTER(_P), C.POINTER(C.c_int32), C.POINTER(C.c_uint64), _D,
                                    C.POINTER(_P)]),
    "mole_batch_destroy": (C.c_int, [_P]),
    "mole_batch_info": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    "mole_batch_init": (C.c_int, [_P, C.c_int32, C.c_double]),
    "mole_batch_set_positions": (C.c_int, [_P, C.c_int32, _D, C.c_int64]),
    "mole_batch_get_positions": (C.c_int, [_P, C.c_int32, _D, C.c_int64]),
    "mole_batch_get_step": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "mole_batch_set_step": (C.c_int, [_P, C.c_uint64]),
    "mole_batch_vmc_run": (C.c_int, [_P, C.POINTER(VmcOpts), _D]),
    "mole_batch_autotune": (C.c_int, [_P, C.POINTER(VmcOpts), C.c_int32, C.POINTER(C.c_int32), _D,
                                      C.POINTER(C.c_int32)]),
    "mole_batch_set_tile": (C.c_int, [_P, C.c_int32]),
    "mole_batch_get_tile": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32]),
    "mole_batch_graph_launches": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "mole_checkpoint_save": (C.c_int, [_P, C.c_char_p]),
    "mole_checkpoint_load": (C.c_int, [_P, C.c_char_p]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libmole_gpu.so; builds it first when absent (nvcc required)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing; run mole_gb300.build.build()")
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.mole_abi_version() != 1:
            raise RuntimeError("libmole_gpu ABI version mismatch")
        _lib = L
        return L


def check(rc: int) -> None:
    if rc != OK:
        msg = load().mole_last_error_string()
        raise MoleError(rc, msg.decode() if msg else "")


def dptr(a):
    return None if a is None else a.ctypes.data_as(_D)
