"""ctypes front end of the CPU FP64 oracle (oracle/mole_oracle.c).

TEST INFRASTRUCTURE ONLY. Imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, and only as the reference the GPU results are
compared with; the product package
never imports it. It accepts any object with the attributes of
``mole_gb300.system.System`` (duck-typed, so the oracle carries no product
code).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

MAX_NUC, MAX_BASIS, MAX_SPIN = 8, 32, 5
MOM_COUNT, MOM_SUM_E, MOM_SUM_E2, MOM_SUM_BLOCK2, MOM_NBLOCKS, MOM_ACCEPT, MOM_PROPOSED, NMOM = range(8)
REF_HELIUM, REF_STO_H, REF_H2_HL, REF_H2ION, REF_GAUSSIAN = range(5)

_lock = threading.Lock()
_libs: dict[str, C.CDLL] = {}


def build() -> None:
    """Compile the oracle and the faithful CPU baseline with the committed Makefile."""
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)


def _load(name: str) -> C.CDLL:
    with _lock:
        if name not in _libs:
            path = os.path.join(BUILD, name)
            if not os.path.exists(path):
                build()
            _libs[name] = C.CDLL(path)
        return _libs[name]


class OrcSystem(C.Structure):
    _fields_ = [
        ("n_nuc", C.c_int32), ("nuc_pos", C.c_double * (MAX_NUC * 3)), ("nuc_z", C.c_int32 * MAX_NUC),
        ("n_up", C.c_int32), ("n_dn", C.c_int32), ("n_basis", C.c_int32),
        ("b_center", C.c_int32 * MAX_BASIS), ("b_kind", C.c_int32 * MAX_BASIS), ("b_exp", C.c_int32 * MAX_BASIS),
        ("n_exp", C.c_int32),
        ("coef_up", C.c_double * (MAX_SPIN * MAX_BASIS)), ("coef_dn", C.c_double * (MAX_SPIN * MAX_BASIS)),
        ("ee_on", C.c_int32), ("ee_npoly", C.c_int32), ("ee_kappa", C.c_double),
        ("cusp_anti", C.c_double), ("cusp_para", C.c_double),
        ("en_on", C.c_int32), ("en_coef", C.c_double * MAX_NUC),
        ("nn_on", C.c_int32), ("pot_kind", C.c_int32), ("omega", C.c_double),
    ]


class OrcEvalOut(C.Structure):
    _fields_ = [("lnpsi", C.c_double), ("sign", C.c_double), ("grad", C.c_double * 30),
                ("lap_over_psi", C.c_double), ("eloc", C.c_double), ("vpot", C.c_double)]


class OrcVmcOpts(C.Structure):
    _fields_ = [("move", C.c_int32), ("step", C.c_double), ("n_eq", C.c_int32), ("n_steps", C.c_int32),
                ("block_size", C.c_int32), ("sr", C.c_int32), ("seed", C.c_uint64), ("step0", C.c_uint32),
                ("walker0", C.c_uint32)]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def to_orc(s) -> OrcSystem:
    o = OrcSystem()
    o.n_nuc = s.n_nuc
    for i in range(s.n_nuc):
        for k in range(3):
            o.nuc_pos[3 * i + k] = float(s.nuc_pos[i, k])
        o.nuc_z[i] = int(s.nuc_z[i])
        o.en_coef[i] = float(s.en_coef[i])
    o.n_up, o.n_dn, o.n_basis, o.n_exp = s.n_up, s.n_dn, s.n_basis, s.n_exp
    for b in range(s.n_basis):
        o.b_center[b] = int(s.basis_center[b])
        o.b_kind[b] = int(s.basis_kind[b])
        o.b_exp[b] = int(s.basis_exp[b])
        for k in range(s.n_up):
            o.coef_up[k * MAX_BASIS + b] = float(s.coef_up[k, b])
        for k in range(s.n_dn):
            o.coef_dn[k * MAX_BASIS + b] = float(s.coef_dn[k, b])
    o.ee_on = int(bool(s.ee_on))
    o.ee_npoly = int(s.ee_poly.size)
    o.ee_kappa = float(s.ee_kappa)
    o.cusp_anti, o.cusp_para = float(s.cusp_anti), float(s.cusp_para)
    o.en_on = int(bool(s.en_on))
    o.nn_on = int(bool(s.nn_on))
    o.pot_kind, o.omega = int(s.pot_kind), float(s.omega)
    return o


def lib() -> C.CDLL:
    L = _load("libmole_oracle.so")
    if not getattr(L, "_typed", False):
        L.orc_num_params.argtypes = [C.POINTER(OrcSystem)]
        L.orc_eval.argtypes = [C.POINTER(OrcSystem), C.POINTER(C.c_double), C.POINTER(C.c_double),
                               C.POINTER(OrcEvalOut), C.POINTER(C.c_double)]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32)] * 3
        L.orc_ref_wf.restype = C.c_double
        L.orc_ref_wf.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_ref_eloc.restype = C.c_double
        L.orc_ref_eloc.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                   C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int, C.c_double]
        L.orc_vmc_run.argtypes = [C.POINTER(OrcSystem), C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double),
                                  C.POINTER(OrcVmcOpts)] + [C.POINTER(C.c_double)] * 5
        L.orc_init_positions.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_double,
                                         C.POINTER(C.c_double)]
        L.orc_dmc_step.restype = C.c_double
        L.orc_dmc_step.argtypes = [C.POINTER(OrcSystem), C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.c_double, C.c_double, C.c_uint64, C.c_uint32,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L._typed = True
    return L


def philox(ctr, key) -> np.ndarray:
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


def num_params(s) -> int:
    o = to_orc(s)
    return lib().orc_num_params(C.byref(o))


def evaluate(s, pos, theta=None, want_O: bool = True) -> dict:
    """lnpsi, sign, grad ln psi, sum_i lap_i psi / psi, E_L, V and O_k for each
    configuration in pos[..., N, 3]."""
    o = to_orc(s)
    th = np.ascontiguousarray(s.params() if theta is None else theta, dtype=np.float64)
    P = th.size
    N = s.n_elec
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, N, 3)
    W = pos.shape[0]
    res = {k: np.zeros(W) for k in ("lnpsi", "sign", "lap", "eloc", "vpot")}
    res["grad"] = np.zeros((W, N, 3))
    res["O"] = np.zeros((W, P))
    out = OrcEvalOut()
    L = lib()
    for w in range(W):
        p = np.ascontiguousarray(pos[w])
        Ow = np.zeros(max(P, 1))
        rc = L.orc_eval(C.byref(o), _dp(th), _dp(p), C.byref(out), _dp(Ow) if want_O else None)
        if rc != 0:
            raise FloatingPointError("singular determinant in oracle")
        res["lnpsi"][w], res["sign"][w] = out.lnpsi, out.sign
        res["lap"][w], res["eloc"][w], res["vpot"][w] = out.lap_over_psi, out.eloc, out.vpot
        res["grad"][w] = np.array(out.grad[:3 * N]).reshape(N, 3)
        res["O"][w] = Ow[:P]
    return res


def init_positions(W: int, N: int, seed: int, kind: int = 0, width: float = 1.0) -> np.ndarray:
    pos = np.zeros((W, N, 3))
    lib().orc_init_positions(W, N, seed, kind, width, _dp(pos))
    return pos


def vmc_run(s, pos, *, move: int, step: float, n_eq: int, n_steps: int, block_size: int, sr: bool = False,
            seed: int = 1, step0: int = 0, theta=None, walker0: int = 0) -> dict:
    """Runs the chains in pos (copied, returned updated) with the GPU path's
    random streams (walker k of pos draws stream walker0 + k); returns
    moments, time-block sums and SR sums."""
    o = to_orc(s)
    th = np.ascontiguousarray(s.params() if theta is None else theta, dtype=np.float64)
    P = th.size
    pos = np.ascontiguousarray(pos, dtype=np.float64).copy()
    W = pos.shape[0]
    opts = OrcVmcOpts(move, step, n_eq, n_steps, block_size, int(sr), seed, step0, walker0)
    mom = np.zeros(NMOM)
    tb = np.zeros(max(n_steps // block_size, 1))
    sO, sEO, sOO = np.zeros(max(P, 1)), np.zeros(max(P, 1)), np.zeros(max(P * P, 1))
    rc = lib().orc_vmc_run(C.byref(o), _dp(th), W, _dp(pos), C.byref(opts), _dp(mom), _dp(tb), _dp(sO),
                           _dp(sEO), _dp(sOO))
    if rc != 0:
        raise FloatingPointError("oracle VMC failed")
    return {"pos": pos, "moments": mom, "time_blocks": tb[: n_steps // block_size], "sum_O": sO[:P],
            "sum_EO": sEO[:P], "sum_OO": sOO[: P * P].reshape(P, P)}


def vmc_run_threads(s, pos, *, threads: int = 0, chunk: int = 4096, **kw) -> dict:
    """vmc_run over a large ensemble, split into slices of `chunk` walkers run
    on host threads (ctypes releases the GIL); every slice keeps its walkers'
    random streams, and the additive sums are added in slice order."""
    from concurrent.futures import ThreadPoolExecutor

    pos = np.ascontiguousarray(pos, dtype=np.float64)
    W = pos.shape[0]
    starts = list(range(0, W, chunk))
    threads = threads or hardware_threads()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(lambda a: vmc_run(s, pos[a:a + chunk], walker0=a, **kw), starts))
    out = {"pos": np.concatenate([p["pos"] for p in parts])}
    for k in ("moments", "time_blocks", "sum_O", "sum_EO", "sum_OO"):
        out[k] = sum(p[k] for p in parts)
    # counts are per walker in the oracle as in the kernels
    return out


def dmc_step(s, pos, eloc, *, tau: float, e_ref: float, seed: int, step: int, theta=None):
    o = to_orc(s)
    th = np.ascontiguousarray(s.params() if theta is None else theta, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64).copy()
    eloc = np.ascontiguousarray(eloc, dtype=np.float64).copy()
    W = pos.shape[0]
    acc, prop = C.c_double(0.0), C.c_double(0.0)
    parent = np.zeros(W, dtype=np.int32)
    ens = lib().orc_dmc_step(C.byref(o), _dp(th), W, _dp(pos), _dp(eloc), tau, e_ref, seed, step, C.byref(acc),
                             C.byref(prop), parent.ctypes.data_as(C.POINTER(C.c_int)))
    return {"pos": pos, "eloc": eloc, "energy": ens, "accepted": acc.value, "proposed": prop.value,
            "parent": parent}


def ref_wf(kind: int, par, pos):
    """psi, grad psi, lap psi, dpsi/dpar of a reference example trial function."""
    par = np.ascontiguousarray(par, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
    g = np.zeros(pos.size)
    lap = C.c_double()
    dp = np.zeros(1)
    v = lib().orc_ref_wf(kind, _dp(par), _dp(pos), _dp(g), C.byref(lap), _dp(dp))
    return v, g.reshape(-1, 3), lap.value, dp[0]


def ref_eloc(kind: int, par, pos, nuc_pos=None, nuc_z=None, harmonic: bool = False, omega: float = 1.0) -> float:
    par = np.ascontiguousarray(par, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
    nuc_pos = np.ascontiguousarray(np.zeros((1, 3)) if nuc_pos is None else nuc_pos, dtype=np.float64)
    nuc_z = np.ascontiguousarray(np.zeros(1) if nuc_z is None else nuc_z, dtype=np.int32)
    return lib().orc_ref_eloc(kind, _dp(par), _dp(pos), nuc_pos.shape[0], _dp(nuc_pos),
                              nuc_z.ctypes.data_as(C.POINTER(C.c_int32)), int(harmonic), omega)


# --------------------------------------------------------- faithful baseline

def faithful_lib() -> C.CDLL:
    L = _load("libmole_faithful.so")
    if not getattr(L, "_typed", False):
        L.faithful_vmc.restype = C.c_double
        L.faithful_vmc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_double)]
        L.faithful_hardware_threads.restype = C.c_int
        L.optimized_vmc.restype = C.c_double
        L.optimized_vmc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                    C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L._typed = True
    return L


def faithful_vmc(system: int, n_walkers: int, n_eq: int, n_steps: int, move: int, step: float, a: float, b: float,
                 sr: bool, threads: int, seed: int = 1):
    """Times the reference's call pattern; returns (seconds, mean energy)."""
    e = C.c_double()
    t = faithful_lib().faithful_vmc(system, n_walkers, n_eq, n_steps, move, step, a, b, int(sr), threads, seed,
                                    C.byref(e))
    return t, e.value


def optimized_vmc(system: int, n_walkers: int, n_eq: int, n_steps: int, step: float, a: float, b: float,
                  threads: int, seed: int = 1):
    """Times the optimised CPU port (cached terms, no allocation); returns
    (seconds, mean energy, acceptance)."""
    e, acc = C.c_double(), C.c_double()
    t = faithful_lib().optimized_vmc(system, n_walkers, n_eq, n_steps, step, a, b, threads, seed, C.byref(e),
                                     C.byref(acc))
    return t, e.value, acc.value


def hardware_threads() -> int:
    return int(faithful_lib().faithful_hardware_threads())
