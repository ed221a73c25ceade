"""Host-side mirror of the reference's plugin surface over the C ABI.

Names, argument meaning and error behaviour follow Jvanrhijn/mole so that code
written against the reference reads the same here, with one difference: every
object works on a whole walker ensemble resident on the GPU instead of one
Array2 configuration.

  reference                                            here
  Function/Differentiate/WaveFunction/Optimize          WaveFunction (a device-side System)
    (src/wavefunction_traits/src/lib.rs:7-24, src/optimize/src/traits.rs:8-16)
  MetropolisBox / MetropolisDiffuse (src/metropolis/src/metrop.rs)   MetropolisBox / MetropolisGaussian / MetropolisDiffuse
  Sampler (src/montecarlo/src/samplers.rs)              Sampler
  Runner::run (src/montecarlo/src/montecarlo.rs:24-46)  Runner.run
  VmcRunner::run_optimization (src/vmc/src/vmc.rs:43-106)    VmcRunner.run_optimization
  SteepestDescent, MomentumDescent, NesterovMomentum, OnlineLbfgs, StochasticReconfiguration
    (src/optimize/src/optimizers.rs)                    same names
  DmcRunner::diffuse (src/dmc/src/dmc.rs:69-202)        DmcRunner.diffuse

Errors raise MoleError whose .kind is the errors::Error variant name.
"""
from __future__ import annotations

import ctypes as C
import math
from collections import deque
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import MoleError, check, dptr
from .system import MOVE_BOX, MOVE_DIFFUSE, MOVE_GAUSS, System

# FP64; FP32 evaluation with FP64 inverse, E_L and sums; FP64-accurate
# double-float on the FP32 pipe (box/Gaussian VMC and evaluation)
PREC_FP64, PREC_MIXED, PREC_DF64 = 0, 1, 2
INIT_NORMAL, INIT_UNIFORM = 0, 1


class Context:
    """One CUDA device; owns device memory and the launch stream."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.mole_ctx_create(device, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.mole_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(self.lib.mole_sync(self.h))

    def set_stream(self, cuda_stream_handle: int | None):
        check(self.lib.mole_ctx_set_stream(self.h, C.c_void_p(cuda_stream_handle or 0)))

    def enable_timing(self, on: bool = True):
        check(self.lib.mole_ctx_enable_timing(self.h, int(on)))

    def kernel_time(self, kernel: int) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_int64()
        check(self.lib.mole_ctx_kernel_time(self.h, kernel, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def df64_reruns(self) -> int:
        """Double-float launches rerun in native FP64 (a value left FP32's exponent range)."""
        n = C.c_int64()
        check(self.lib.mole_ctx_df64_reruns(self.h, C.byref(n)))
        return n.value

    def math_check(self, fn: int, x) -> np.ndarray:
        """The library's device arithmetic on x (0: FP64 exp of the native kernels,
        1-4: double-float exp, rsqrt, reciprocal, x / (1 + x^2); 5, 6: the
        integer-built float -> double and double -> float (toward zero)
        conversions; 7: the latter for magnitudes below FP32's largest; 8, 9: the
        FP64 reciprocal and reciprocal square root of the native kernels)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        check(self.lib.mole_math_check(self.h, fn, dptr(x), x.size, dptr(y)))
        return y

    def probe_peaks(self) -> tuple[float, float]:
        """(FP64, FP32) FMA GFLOP/s measured on this device."""
        a, b = C.c_double(), C.c_double()
        check(self.lib.mole_probe_peaks(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value


class WaveFunction:
    """Device-side Slater-Jastrow wavefunction with its Hamiltonian; the
    Function + Differentiate + WaveFunction + Optimize surface of the reference."""

    def __init__(self, ctx: Context, system: System):
        self.ctx, self.lib, self.system = ctx, ctx.lib, system
        s = system
        self._keep = dict(
            nuc_pos=np.ascontiguousarray(s.nuc_pos, dtype=np.float64), nuc_z=np.ascontiguousarray(s.nuc_z, np.int32),
            bc=np.ascontiguousarray(s.basis_center, np.int32), bk=np.ascontiguousarray(s.basis_kind, np.int32),
            be=np.ascontiguousarray(s.basis_exp, np.int32), cu=np.ascontiguousarray(s.coef_up, np.float64),
            cd=np.ascontiguousarray(s.coef_dn if s.n_dn else np.zeros((1, s.n_basis)), np.float64),
            en=np.ascontiguousarray(s.en_coef, np.float64))
        k = self._keep
        i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
        d = _lib.SystemDesc(s.n_nuc, dptr(k["nuc_pos"]), i32(k["nuc_z"]), s.n_up, s.n_dn, s.n_basis, i32(k["bc"]),
                            i32(k["bk"]), i32(k["be"]), s.n_exp, dptr(k["cu"]), dptr(k["cd"]), int(s.ee_on),
                            int(s.ee_poly.size), s.ee_kappa, s.cusp_anti, s.cusp_para, int(s.en_on), dptr(k["en"]),
                            int(s.nn_on), s.pot_kind, s.omega)
        th = s.params()
        h = C.c_void_p()
        check(self.lib.mole_system_create(ctx.h, C.byref(d), dptr(th), th.size, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.mole_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_electrons(self) -> int:
        return self.system.n_elec

    def num_parameters(self) -> int:
        n = C.c_int32()
        check(self.lib.mole_num_params(self.h, C.byref(n)))
        return n.value

    def parameters(self) -> np.ndarray:
        th = np.zeros(self.num_parameters())
        check(self.lib.mole_params_get(self.h, dptr(th), th.size))
        return th

    def set_parameters(self, theta) -> None:
        th = np.ascontiguousarray(theta, dtype=np.float64)
        check(self.lib.mole_params_set(self.h, dptr(th), th.size))
        self.system = self.system.with_params(th)

    def update_parameters(self, deltap) -> None:
        """Optimize::update_parameters: theta += deltap."""
        self.set_parameters(self.parameters() + np.asarray(deltap, dtype=np.float64))


class Walkers:
    """A walker ensemble resident on the device."""

    def __init__(self, wf: WaveFunction, n_walkers: int, seed: int = 0x5EED, init: int = INIT_NORMAL,
                 width: float = 1.0):
        self.wf, self.lib = wf, wf.lib
        h = C.c_void_p()
        check(self.lib.mole_walkers_create(wf.h, n_walkers, seed, C.byref(h)))
        self.h = h
        self.n = n_walkers
        if init != INIT_NORMAL or width != 1.0:
            self.init(init, width)

    def close(self):
        if self.h:
            self.lib.mole_walkers_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, kind: int = INIT_NORMAL, width: float = 1.0):
        check(self.lib.mole_walkers_init(self.h, kind, width))

    @property
    def shape(self):
        return (self.n, self.wf.num_electrons(), 3)

    def positions(self) -> np.ndarray:
        p = np.zeros(self.shape)
        check(self.lib.mole_walkers_get_positions(self.h, dptr(p), p.size))
        return p

    def set_positions(self, pos) -> None:
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(self.shape)
        check(self.lib.mole_walkers_set_positions(self.h, dptr(p), p.size))

    @property
    def step(self) -> int:
        s = C.c_uint64()
        check(self.lib.mole_walkers_get_step(self.h, C.byref(s)))
        return s.value

    @step.setter
    def step(self, v: int):
        check(self.lib.mole_walkers_set_step(self.h, int(v)))

    def evaluate(self, precision: int = PREC_FP64, want_O: bool = True) -> dict:
        """lnpsi, sign, grad ln psi, sum_i lap_i psi/psi, E_L and O_k at the current positions."""
        W, N, P = self.n, self.wf.num_electrons(), self.wf.num_parameters()
        r = {"lnpsi": np.zeros(W), "sign": np.zeros(W), "grad": np.zeros((W, N, 3)), "lap": np.zeros(W),
             "eloc": np.zeros(W), "O": np.zeros((W, P)) if want_O else None}
        check(self.lib.mole_eval(self.h, precision, dptr(r["lnpsi"]), dptr(r["sign"]), dptr(r["grad"]),
                                 dptr(r["lap"]), dptr(r["eloc"]), dptr(r["O"])))
        return r

    # --- stochastic reconfiguration with many parameters (the neural Jastrow)
    def sr_collect_begin(self):
        check(self.lib.mole_sr_collect_begin(self.h))

    def sr_collect_sample(self, precision: int = PREC_MIXED):
        check(self.lib.mole_sr_collect_sample(self.h, precision))

    def sr_collect_solve(self, eps: float, step: float, max_iter: int = 500, tol: float = 1e-8):
        P = self.wf.num_parameters()
        delta, g, info = np.zeros(P), np.zeros(P), np.zeros(4)
        check(self.lib.mole_sr_collect_solve(self.h, eps, step, max_iter, tol, dptr(delta), dptr(g), dptr(info)))
        return delta, g, info

    def sr_collect_matrix(self, eps: float) -> np.ndarray:
        P = self.wf.num_parameters()
        S = np.zeros((P, P))
        check(self.lib.mole_sr_collect_matrix(self.h, eps, dptr(S)))
        return S

    def save(self, path: str):
        check(self.lib.mole_checkpoint_save(self.h, path.encode()))

    def load(self, path: str):
        check(self.lib.mole_checkpoint_load(self.h, path.encode()))
        self.wf.system = self.wf.system.with_params(self.wf.parameters())


# ------------------------------------------------------------------- moves

@dataclass
class MetropolisBox:
    """Uniform cube of side box_side around the electron (metrop.rs:22-101)."""
    box_side: float
    kind: int = MOVE_BOX

    @property
    def step(self):
        return self.box_side


@dataclass
class MetropolisGaussian:
    """Isotropic Gaussian single-electron move of width sigma, symmetric acceptance."""
    sigma: float
    kind: int = MOVE_GAUSS

    @property
    def step(self):
        return self.sigma


@dataclass
class MetropolisDiffuse:
    """Drift-diffusion move with the all-electron Green's-function ratio and
    node-crossing rejection (metrop.rs:104-217)."""
    time_step: float
    kind: int = MOVE_DIFFUSE

    @property
    def step(self):
        return self.time_step


# ------------------------------------------------------------- statistics

def blocking_error(moments) -> float:
    """Blocking error sqrt((<B^2> - E^2)/(n_b - 1)) of src/vmc/src/vmc.rs:158-167,
    blocks being consecutive block_size samples of one chain."""
    nb = moments[4]
    if nb < 2:
        return float("nan")
    mean = moments[1] / moments[0]
    b2 = moments[3] / nb
    return math.sqrt(max(b2 - mean * mean, 0.0) / (nb - 1.0))


@dataclass
class MonteCarloResult:
    """MonteCarloResult (src/montecarlo/src/traits.rs:5-10) reduced on the device."""
    energy: float
    error: float
    variance: float
    acceptance: float
    moments: np.ndarray
    time_blocks: np.ndarray
    sum_O: np.ndarray | None = None
    sum_EO: np.ndarray | None = None
    sum_OO: np.ndarray | None = None

    @property
    def count(self) -> float:
        return float(self.moments[0])

    def energy_gradient(self) -> np.ndarray:
        """compute_energy_gradient (src/optimize/src/util.rs:6-46) with O_k = d ln psi/d p_k:
        g_k = 2 (<E O_k> - <E><O_k>)."""
        n = self.count
        return 2.0 * (self.sum_EO / n - self.energy * self.sum_O / n)


@dataclass
class ObservableResult:
    """Per-observable means over walkers and samples, with the blocking error
    of the per-sample ensemble means (src/vmc/src/vmc.rs:133-172)."""
    mean: dict
    error: dict
    samples: int


class Sampler:
    """Sampler (src/montecarlo/src/samplers.rs): a wavefunction, a move and an ensemble."""

    def __init__(self, wave_function: WaveFunction, metropolis, walkers: Walkers, precision: int = PREC_FP64,
                 refresh: int = 100):
        self.wf, self.metropolis, self.walkers = wave_function, metropolis, walkers
        self.precision, self.refresh = precision, refresh

    def wave_function(self) -> WaveFunction:
        return self.wf

    def run(self, n_eq: int, n_steps: int, block_size: int, sr: bool = False) -> MonteCarloResult:
        lib = self.wf.lib
        P = self.wf.num_parameters()
        o = _lib.VmcOpts(self.metropolis.kind, self.metropolis.step, n_eq, n_steps, block_size, int(sr),
                         self.precision, self.refresh)
        mom = np.zeros(_lib.NMOM)
        tb = np.zeros(max(n_steps // block_size, 1))
        sO = np.zeros(P) if sr else None
        sEO = np.zeros(P) if sr else None
        sOO = np.zeros((P, P)) if sr else None
        check(lib.mole_vmc_run(self.walkers.h, C.byref(o), dptr(mom), dptr(tb), dptr(sO), dptr(sEO), dptr(sOO)))
        n = mom[0]
        E = mom[1] / n if n else float("nan")
        var = mom[2] / n - E * E if n else float("nan")
        return MonteCarloResult(E, blocking_error(mom), var, mom[5] / max(mom[6], 1.0), mom, tb[: n_steps // block_size],
                                sO, sEO, sOO)

    def sample_observables(self, observables: dict, n_samples: int, every: int = 1,
                           block_size: int = 1) -> ObservableResult:
        """Sampler::sample with user observables (src/montecarlo/src/samplers.rs:81-104):
        every `every` sweeps the walkers' positions and log-form evaluation are
        handed to each LocalOperator (mole_gb300.operators) and its walker mean
        recorded; returns the means over samples and their blocking errors
        (blocks of `block_size` samples)."""
        from .operators import WalkerBatch

        wk = self.walkers
        want_O = any(getattr(o, "needs_O", False) for o in observables.values())
        series = {k: [] for k in observables}
        for _ in range(n_samples):
            self.run(every, 0, 1)
            ev = wk.evaluate(self.precision, want_O=want_O)
            b = WalkerBatch(wk.positions(), ev["lnpsi"], ev["sign"], ev["grad"], ev["lap"], ev["eloc"], ev["O"])
            for k, op in observables.items():
                series[k].append(np.mean(np.asarray(op.act_on(b), dtype=np.float64), axis=0))
        mean, err = {}, {}
        for k, v in series.items():
            x = np.array(v)
            mean[k] = x.mean(axis=0)
            nb = len(x) // block_size
            if nb > 1:
                bm = x[: nb * block_size].reshape((nb, block_size) + x.shape[1:]).mean(axis=1)
                err[k] = np.sqrt(np.maximum((bm * bm).mean(axis=0) - bm.mean(axis=0) ** 2, 0.0) / (nb - 1))
            else:
                err[k] = np.full(np.shape(mean[k]), np.nan)
        return ObservableResult(mean, err, n_samples)


class Runner:
    """Runner (src/montecarlo/src/montecarlo.rs:24-46): steps/block_size blocks,
    block 0 discarded as equilibration, one sample per sweep afterwards."""

    def __init__(self, sampler: Sampler):
        self.sampler = sampler

    def run(self, steps: int, block_size: int, sr: bool = False) -> MonteCarloResult:
        if steps < 2 * block_size:
            raise MoleError(2, "steps must be at least 2 * block_size")
        blocks = steps // block_size
        return self.sampler.run(block_size, (blocks - 1) * block_size, block_size, sr=sr)


# -------------------------------------------------------------- optimizers

class SteepestDescent:
    """optimizers.rs:9-43: delta = -step * g."""

    def __init__(self, step_size: float):
        self.step_size = step_size

    def compute_parameter_update(self, pars, result: MonteCarloResult, ctx: Context | None = None):
        return -self.step_size * result.energy_gradient()


class MomentumDescent:
    """optimizers.rs:45-73: m -= step * g; delta = mu * m."""

    def __init__(self, step_size: float, momentum_parameter: float, nparm: int):
        self.step_size, self.mu = step_size, momentum_parameter
        self.momentum = np.zeros(nparm)

    def compute_parameter_update(self, pars, result, ctx=None):
        self.momentum -= self.step_size * result.energy_gradient()
        return self.mu * self.momentum


class NesterovMomentum:
    """optimizers.rs:75-107."""

    def __init__(self, step_size: float, momentum_parameter: float, nparm: int):
        self.step_size, self.mu = step_size, momentum_parameter
        self.momentum = np.zeros(nparm)
        self.momentum_prev = np.zeros(nparm)

    def compute_parameter_update(self, pars, result, ctx=None):
        g = result.energy_gradient()
        self.momentum_prev = self.momentum.copy()
        self.momentum = self.mu * self.momentum + self.step_size * g
        return -(self.mu * self.momentum_prev + (1.0 + self.mu) * self.momentum)


class OnlineLbfgs:
    """optimizers.rs:109-192 (online L-BFGS two-loop recursion)."""

    def __init__(self, step_size: float, history: int, nparm: int):
        eps = 1e-5
        self.step_size, self.history = step_size, history
        self.grad_prev = np.full(nparm, eps)
        self.pars_prev = np.full(nparm, eps)
        self.s: deque = deque()
        self.y: deque = deque()
        self.iter = 0

    def _initial_direction(self, g):
        p = -g
        alphas = []
        for s, y in zip(reversed(self.s), reversed(self.y)):
            a = s.dot(p) / s.dot(y)
            p = p - a * y
            alphas.append(a)
        if self.iter == 0:
            p = p * 1e-10
        else:
            p = p * sum(s.dot(y) / y.dot(y) for s, y in zip(self.s, self.y)) / min(self.iter, self.history)
        for a, s, y in zip(reversed(alphas), self.s, self.y):
            p = p + (a - y.dot(p) / y.dot(s)) * s
        return p

    def _update_pairs(self, pars, g):
        if len(self.s) >= self.history:
            self.s.popleft()
        self.s.append(pars - self.pars_prev)
        if len(self.y) >= self.history:
            self.y.popleft()
        self.y.append(g - self.grad_prev)

    def compute_parameter_update(self, pars, result, ctx=None):
        g = result.energy_gradient()
        self._update_pairs(pars, g)
        p = self._initial_direction(g)
        s = -self.step_size * p
        self._update_pairs(pars, g)
        self.grad_prev, self.pars_prev = g.copy(), np.array(pars, dtype=np.float64)
        self.iter += 1
        return s


class StochasticReconfiguration:
    """optimizers.rs:194-265 with O_k = d ln psi / d p_k, S_kl = <O_k O_l> - <O_k><O_l>,
    S_kk += eps and delta = step * S^-1 (-g/2), solved in FP64 on the device side.
    With more than 8 parameters (the neural Jastrow) the sums are not
    accumulated per walker: VmcRunner takes `samples` O_k samples of the whole
    ensemble per iteration, `sample_every` sweeps apart, and S is built on the
    tensor cores and solved by conjugate gradients."""

    def __init__(self, step_size: float, eps: float = 1e-3, samples: int = 8, sample_every: int = 10,
                 precision: int = PREC_MIXED, max_iter: int = 500):
        self.step_size, self.eps = step_size, eps
        self.samples, self.sample_every, self.precision = samples, sample_every, precision
        self.max_iter = max_iter
        self.last_info = None

    def collect_and_solve(self, sampler: "Sampler"):
        wk = sampler.walkers
        wk.sr_collect_begin()
        for _ in range(self.samples):
            sampler.run(0, self.sample_every, self.sample_every)
            wk.sr_collect_sample(self.precision)
        try:
            delta, g, info = wk.sr_collect_solve(self.eps, self.step_size, max_iter=self.max_iter)
        except MoleError as e:
            # an ill-conditioned S (late in a long training) can need more CG
            # iterations: one retry with four times as many, then the error
            if e.kind != "LinalgError":
                raise
            delta, g, info = wk.sr_collect_solve(self.eps, self.step_size, max_iter=4 * self.max_iter)
        self.last_info = info
        return delta, g

    def compute_parameter_update(self, pars, result: MonteCarloResult, ctx: Context):
        P = result.sum_O.size
        delta, g = np.zeros(P), np.zeros(P)
        sE = np.array([result.moments[1]])
        check(ctx.lib.mole_sr_update(ctx.h, P, result.count, dptr(sE), dptr(result.sum_O), dptr(result.sum_EO),
                                     dptr(np.ascontiguousarray(result.sum_OO)), self.eps, self.step_size,
                                     dptr(delta), dptr(g)))
        return delta


class VmcRunner:
    """VmcRunner::run_optimization (src/vmc/src/vmc.rs:43-106). Each iteration
    runs every walker for `steps` sweeps with the first block discarded,
    reduces energy, blocking error and the O_k sums on the device, and applies
    the optimizer's update to the wavefunction. Unlike the reference, the
    chains continue from where the previous iteration left them."""

    def __init__(self, sampler: Sampler, optimizer, group=None):
        self.sampler, self.optimizer = sampler, optimizer
        self.group = group  # torch.distributed group whose ranks split the walkers (None: all ranks)

    def run_optimization(self, iters: int, steps: int, block_size: int, callback=None):
        from .distributed import allreduce_result, world

        wf = self.sampler.wave_function()
        energies, errors, results = [], [], []
        large = wf.num_parameters() > 8
        multi = world()[1] > 1
        if multi and large:
            raise MoleError(103, "the many-parameter SR path runs on one rank")
        for it in range(iters):
            r = Runner(self.sampler).run(steps, block_size, sr=not large)
            if multi:  # every rank's sums, so every rank takes the same step
                r = allreduce_result(r, self.group)
            energies.append(r.energy)
            errors.append(r.error)
            results.append(r)
            if large:
                if not isinstance(self.optimizer, StochasticReconfiguration):
                    raise MoleError(103, "only StochasticReconfiguration handles more than 8 parameters")
                delta, _ = self.optimizer.collect_and_solve(self.sampler)
            else:
                delta = self.optimizer.compute_parameter_update(wf.parameters(), r, wf.ctx)
            wf.update_parameters(delta)
            if callback:
                callback(it, r, wf)
        return wf, np.array(energies), np.array(errors), results


# --------------------------------------------------------------------- DMC

class DmcRunner:
    """DmcRunner (src/dmc/src/dmc.rs:16-202): drift-diffusion with Metropolis,
    weights exp(-tau((E_L + E_L')/2 - E_ref)) and, every step, a stochastic
    comb in place of SRBrancher (constant population, equal weights).

    The move is the reference's MetropolisDiffuse (src/metropolis/src/metrop.rs:150-198),
    whose Green's-function ratio includes the drift of every electron: next to
    a node the unmoved partner's drift (~1/distance) drives the reverse factor
    to zero and any proposal is accepted, so a walker can be thrown far out. A
    walker whose Slater matrix is singular at its orbitals' precision (on a
    node, or with every orbital of an electron underflowed) gets zero weight,
    is left out of that step's energy and is removed by the comb; node_kills
    counts them."""

    def __init__(self, guiding_wave_function: WaveFunction, walkers: Walkers, reference_energy: float,
                 precision: int = PREC_FP64, eloc_cutoff: float = 0.0):
        self.wf, self.walkers = guiding_wave_function, walkers
        self.reference_energy = reference_energy
        self.precision = precision
        # 0: the raw E_L in the weights (the reference's DMC); > 0: clipped to
        # reference_energy +- eloc_cutoff in the weight factor only
        self.eloc_cutoff = eloc_cutoff
        self.accepted = 0.0
        self.proposed = 0.0
        self.step_energies: list[np.ndarray] = []

    def run_block(self, time_step: float, n_steps: int) -> np.ndarray:
        o = _lib.DmcOpts(time_step, self.reference_energy, n_steps, self.precision, 0, self.eloc_cutoff)
        e = np.zeros(n_steps)
        acc = np.zeros(2)
        check(self.wf.lib.mole_dmc_run(self.walkers.h, C.byref(o), dptr(e), dptr(acc)))
        self.accepted += acc[0]
        self.proposed += acc[1]
        self.step_energies.append(e)
        return e

    def diffuse(self, time_step: float, num_iterations: int, block_size: int, num_eq_blocks: int):
        """Returns (energies, errors) with the running estimates of
        update_energies (dmc.rs:155-202)."""
        energies: list[float] = []
        variances: list[float] = []
        for block_nr in range(num_iterations // block_size):
            e = self.run_block(time_step, block_size)
            energy = float(e.mean())
            if block_nr == num_eq_blocks:
                self.reference_energy = (self.reference_energy + energy) / 2.0
                energies.append(energy)
                variances.append(0.0)
            elif block_nr > num_eq_blocks:
                k = block_nr - num_eq_blocks
                prev = energies[-1]
                energies.append(prev + (energy - prev) / k)
                self.reference_energy = (self.reference_energy + energies[-1]) / 2.0
                variances.append(variances[-1] + ((energy - prev) * (energy - energies[-1]) - variances[-1]) / k)
        errors = [math.sqrt(v / (i + 1)) for i, v in enumerate(variances)]
        return np.array(energies), np.array(errors)

    @property
    def acceptance(self) -> float:
        return self.accepted / max(self.proposed, 1.0)

    @property
    def node_kills(self) -> float:
        """Walkers found on a node of the guide (psi = 0 at the orbitals'
        precision) and given zero weight, over this walker set's DMC steps."""
        k = C.c_double()
        check(self.wf.lib.mole_dmc_node_kills(self.walkers.h, C.byref(k)))
        return k.value


# ------------------------------------------------------------------ batches

def _tile_cache_path() -> str:
    import os

    return os.environ.get("MOLE_GB300_TILE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "mole_gb300", "batch_tiles.json"))


class Batch:
    """A ragged batch of independent systems (each with its own walker
    ensemble, electron count up to 5 + 5 and parameters) advanced by one
    persistent launch replayed as a CUDA graph. It stands where the reference
    runs Runner::run once per system and chain (src/montecarlo/src/montecarlo.rs:24-46,
    src/vmc/src/vmc.rs:63-76).

    ``systems`` are System descriptors or WaveFunctions; ``seeds[k]`` keys
    system k's random streams exactly as ``Walkers(wf, W, seed)`` does;
    ``widths[k]`` is system k's proposal width, multiplied by the move's step
    at run time."""

    def __init__(self, ctx: Context, systems, n_walkers, seeds=None, widths=None):
        self.ctx, self.lib = ctx, ctx.lib
        self.wfs = [s if isinstance(s, WaveFunction) else WaveFunction(ctx, s) for s in systems]
        S = len(self.wfs)
        self.n_walkers = np.ascontiguousarray(n_walkers, dtype=np.int32).reshape(S)
        sd = np.arange(S, dtype=np.uint64) + np.uint64(0x5EED) if seeds is None else seeds
        self.seeds = np.ascontiguousarray(sd, dtype=np.uint64).reshape(S)
        self.widths = None if widths is None else np.ascontiguousarray(widths, dtype=np.float64).reshape(S)
        hs = (C.c_void_p * S)(*[wf.h.value for wf in self.wfs])
        h = C.c_void_p()
        check(self.lib.mole_batch_create(ctx.h, S, hs, self.n_walkers.ctypes.data_as(C.POINTER(C.c_int32)),
                                         self.seeds.ctypes.data_as(C.POINTER(C.c_uint64)), dptr(self.widths),
                                         C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.mole_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self) -> int:
        return len(self.wfs)

    @property
    def total_walkers(self) -> int:
        return int(self.n_walkers.sum())

    def electrons(self, k: int) -> int:
        return self.wfs[k].num_electrons()

    def init(self, kind: int = INIT_NORMAL, width: float = 1.0):
        check(self.lib.mole_batch_init(self.h, kind, width))

    def positions(self, k: int) -> np.ndarray:
        p = np.zeros((int(self.n_walkers[k]), self.electrons(k), 3))
        check(self.lib.mole_batch_get_positions(self.h, k, dptr(p), p.size))
        return p

    def set_positions(self, k: int, pos) -> None:
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(int(self.n_walkers[k]), self.electrons(k), 3)
        check(self.lib.mole_batch_set_positions(self.h, k, dptr(p), p.size))

    @property
    def step(self) -> int:
        s = C.c_uint64()
        check(self.lib.mole_batch_get_step(self.h, C.byref(s)))
        return s.value

    @step.setter
    def step(self, v: int):
        check(self.lib.mole_batch_set_step(self.h, int(v)))

    def _opts(self, metropolis, n_eq, n_steps, block_size, precision, refresh):
        return _lib.VmcOpts(metropolis.kind, metropolis.step, n_eq, n_steps, block_size, 0, precision, refresh)

    def run(self, metropolis, n_eq: int, n_steps: int, block_size: int, precision: int = PREC_MIXED,
            refresh: int = 100) -> list[MonteCarloResult]:
        """One graph replay: n_eq + n_steps sweeps of every system; a
        MonteCarloResult per system."""
        o = self._opts(metropolis, n_eq, n_steps, block_size, precision, refresh)
        mom = np.zeros((len(self), _lib.NMOM))
        check(self.lib.mole_batch_vmc_run(self.h, C.byref(o), dptr(mom)))
        out = []
        for m in mom:
            n = m[0]
            E = m[1] / n if n else float("nan")
            var = m[2] / n - E * E if n else float("nan")
            out.append(MonteCarloResult(E, blocking_error(m), var, m[5] / max(m[6], 1.0), m, np.zeros(0)))
        return out

    @property
    def tile(self) -> int:
        w, c = C.c_int32(), C.c_int32()
        check(self.lib.mole_batch_get_tile(self.h, C.byref(w), C.byref(c), PREC_MIXED))
        return w.value

    @tile.setter
    def tile(self, walkers_per_cta: int):
        check(self.lib.mole_batch_set_tile(self.h, int(walkers_per_cta)))

    def grid(self, precision: int = PREC_MIXED) -> int:
        w, c = C.c_int32(), C.c_int32()
        check(self.lib.mole_batch_get_tile(self.h, C.byref(w), C.byref(c), precision))
        return c.value

    @property
    def graph_launches(self) -> int:
        n = C.c_int64()
        check(self.lib.mole_batch_graph_launches(self.h, C.byref(n)))
        return n.value

    def tile_key(self, metropolis, precision: int) -> str:
        """Cache key of a tuned tile: device (SMs, compute capability),
        precision, move and the batch's largest spin blocks, electron-count
        profile and total walkers (to a power of two)."""
        n_sm, ma, mi = C.c_int32(), C.c_int32(), C.c_int32()
        check(self.lib.mole_ctx_device_info(self.ctx.h, C.byref(n_sm), C.byref(ma), C.byref(mi)))
        ns = sorted({self.electrons(k) for k in range(len(self))})
        tot = 1 << max(int(self.total_walkers) - 1, 0).bit_length()
        return f"sm{ma.value}{mi.value}x{n_sm.value}|p{precision}|m{metropolis.kind}|N{','.join(map(str, ns))}|W{tot}"

    def autotune(self, metropolis, precision: int = PREC_MIXED, sweeps: int = 10, cache: bool = True) -> dict:
        """Picks the walkers-per-CTA tile by timing every candidate on a copy of
        the positions (the chains are untouched); with ``cache`` a tile tuned
        before for the same key is reused from the JSON tile cache."""
        import json
        import os

        key = self.tile_key(metropolis, precision)
        path = _tile_cache_path()
        table = {}
        if cache and os.path.exists(path):
            try:
                with open(path) as f:
                    table = json.load(f)
            except (OSError, ValueError):
                table = {}
            if key in table:
                self.tile = int(table[key]["tile"])
                return {"tile": self.tile, "cached": True, "key": key, "timings": table[key].get("timings", {})}
        o = self._opts(metropolis, 0, sweeps, sweeps, precision, 100)
        wpb, ms, n = (C.c_int32 * 8)(), (C.c_double * 8)(), C.c_int32()
        check(self.lib.mole_batch_autotune(self.h, C.byref(o), 8, wpb, ms, C.byref(n)))
        timings = {int(wpb[i]): float(ms[i]) for i in range(n.value)}
        res = {"tile": self.tile, "cached": False, "key": key, "timings": timings}
        if cache:
            table[key] = {"tile": res["tile"], "timings": {str(k): v for k, v in timings.items()}}
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                with open(path + ".tmp", "w") as f:
                    json.dump(table, f, indent=1, sort_keys=True)
                os.replace(path + ".tmp", path)
            except OSError:
                pass
        return res


def ragged_batch(n_systems: int = 256, rng: np.random.Generator | None = None, w_range=(256, 4096),
                 z_range=(2, 10), n_range=(2, 10)):
    """The ragged-batch workload: n_systems atoms/ions from ``random_atom``
    (Z in U{2..10}, N in U{2..10}, 1s/2s/2p STOs with exponents U[0.5, Z],
    Pade e-e and e-n Jastrows), walker counts U{256..4096}, a Gaussian
    proposal width 0.6 / sqrt(Z) each. Returns (systems, walkers, widths)."""
    from .system import random_atom

    rng = rng or np.random.default_rng(0x5EED + 2)
    systems = [random_atom(rng, z_range=z_range, n_range=n_range) for _ in range(n_systems)]
    walkers = rng.integers(w_range[0], w_range[1] + 1, size=n_systems)
    widths = np.array([0.6 / math.sqrt(float(s.nuc_z[0])) for s in systems])
    return systems, walkers, widths
