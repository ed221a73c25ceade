"""Algorithmic floating-point work of the walker kernels, per walker-step.

A walker-step is one sweep of N single-electron proposals with accept/reject,
one local-energy evaluation and (when SR is on) the O_k accumulation. Counts
follow the formulas the kernels evaluate (mole_gb300/csrc/walker.cuh):
add, multiply and compare-free arithmetic count 1, a fused multiply-add 2;
exp, log, sqrt, rsqrt, sincos and division count 1 each and are also
tallied separately as "special" operations, which the FP64 pipe expands into
many instructions. The Sherman-Morrison update is weighted by the measured
acceptance ratio.
"""
from __future__ import annotations

from dataclasses import dataclass

from .system import GTO_1S, MOVE_BOX, MOVE_DIFFUSE, MOVE_GAUSS, STO_1S, System


@dataclass
class Work:
    flops: float = 0.0
    special: float = 0.0

    def add(self, f: float, s: float = 0.0) -> "Work":
        self.flops += f
        self.special += s
        return self


def _basis_counts(system: System, spin_n: int, grad: bool, lap: bool, dz: bool) -> Work:
    """One electron: distances to every nucleus, every basis function, the
    orbital accumulation for spin_n orbitals, e-n Jastrow and potential."""
    w = Work()
    for I in range(system.n_nuc):
        w.add(3 + 5 + 1, 1)  # displacement, r^2, r from rsqrt
        if lap:
            w.add(2)  # -Z / r
        for b in range(system.n_basis):
            if system.basis_center[b] != I:
                continue
            kind = int(system.basis_kind[b])
            w.add(2, 1)  # exponent argument and exp
            if kind == STO_1S:
                kf = (3 + 3 if grad else 0) + (4 if lap else 0)
            elif kind == GTO_1S:
                kf = (2 + 3 if grad else 0) + (5 if lap else 0)
            else:
                kf = 1 + (4 + 3 if grad else 0) + (5 if lap else 0)
            w.add(kf + 2 * spin_n * (1 + (3 if grad else 0) + (1 if lap else 0)))
            if dz:
                w.add(2 * spin_n + 4)
        if system.en_on:
            w.add(5 + (4 if grad else 0) + (7 if lap else 0) + (5 if dz else 0), 1)
    return w


def _pair_counts(system: System, deriv: bool, par: bool) -> Work:
    w = Work().add(3 + 5 + 1, 1)
    if system.ee_on:
        w.add(2 + 2, 1)  # q = 1/(1 + b r), u
        if system.ee_kappa > 0:
            w.add(4, 1)
        w.add(4 * system.ee_poly.size)
        if deriv:
            w.add(6 + 9 + 4)  # u', u'', gradient and Laplacian accumulation
        if par:
            w.add(4 + 2 * system.ee_poly.size)
    return w


def walker_step(system: System, move: int, sr_params: int = 0, acceptance: float = 0.5) -> Work:
    N = system.n_elec
    w = Work()
    for e in range(N):
        n = system.n_up if e < system.n_up else system.n_dn
        # proposal
        if move == MOVE_BOX:
            w.add(14)
        else:
            w.add(21, 6)
            if move == MOVE_DIFFUSE:
                w.add(6, 1)
        w.add(3)  # new position
        drift = move == MOVE_DIFFUSE
        w.flops += _basis_counts(system, n, drift, False, False).flops
        w.special += _basis_counts(system, n, drift, False, False).special
        w.add(2 * n)  # determinant ratio
        for _ in range(N - 1):
            p = _pair_counts(system, drift, False)
            w.add(p.flops + 2, p.special)
            if drift:  # old-pair derivative for the drift update
                w.add(p.flops, p.special)
        w.add(3, 1)  # acceptance probability
        if drift:
            w.add(4 * n * n + 2 * n + 6 * N * n + 12 * N + 12 * N, 1)  # tentative inverse, drifts, G ratio
        w.add(acceptance * (4 * n * n + 2 * n), acceptance)  # Sherman-Morrison update
    # local energy
    for e in range(N):
        n = system.n_up if e < system.n_up else system.n_dn
        b = _basis_counts(system, n, True, True, sr_params > 0)
        w.add(b.flops + 8 * n + 20, b.special)
    pairs = N * (N - 1) // 2
    p = _pair_counts(system, True, sr_params > 0)
    w.add(pairs * (p.flops + 1), pairs * p.special)
    w.add(3 + 2)  # assembly and potential constant
    # accumulation: E, E^2, blocking, O_k, E O_k, O_k O_l
    w.add(4 + 2 * sr_params + sr_params * (sr_params + 1))
    return w


def batch_step_fp64(n_up: int, n_dn: int, acceptance: float = 0.5) -> Work:
    """FP64 arithmetic of one walker-step of the ragged-batch kernel in its
    FP32-evaluation form (mole_gb300/csrc/batch.cuh): per move the
    determinant ratio (n products), on acceptance the Sherman-Morrison
    row update (v = phi B, B -= col v^T, one division) and the FP64 position
    update; per electron of the local energy the gradient and Laplacian
    contractions with the inverse (4 n products), the dot product with the
    Jastrow gradient and the assembly. Orbital, Jastrow and potential terms
    are FP32 work and are not counted here."""
    w = Work()
    for e in range(n_up + n_dn):
        n = n_up if e < n_up else n_dn
        w.add(2 * n)
        w.add(acceptance * (4 * n * n + n + 3), acceptance)
        w.add(8 * n + 6 + 4)
    w.add(4)  # E, E^2 and blocking sums
    return w
