"""Local operators: the reference's LocalOperator<T> observables over a
device-resident ensemble.

The reference samples every observable as act_on(psi, cfg) / psi per walker
and step (src/operator/src/traits.rs:262-265, src/montecarlo/src/samplers.rs:81-104).
A trait object cannot run inside the sweep kernel, so an observable here is a
host callback on a batch of walkers: `act_on(batch)` returns O psi / psi for
every walker, where `batch` carries the walkers' positions [W][N][3] and what
the device evaluated there in log form -- ln|psi|, sign, grad ln psi,
sum_i lap_i psi / psi, E_L and, when asked for, O_k = d ln psi / d theta_k.
Sampler.sample_observables runs the sweeps on the device and hands such a
batch to every observable every `every` sweeps.

Built-in operators follow src/operator/src/operator.rs and
src/vmc/src/operators.rs; HarmonicPotential and HarmonicHamiltonian are the
user-defined operator of examples/custom_operator.rs:29-61.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class WalkerBatch:
    """Positions and the device's log-form evaluation at them."""
    pos: np.ndarray        # [W][N][3]
    lnpsi: np.ndarray      # [W]
    sign: np.ndarray       # [W]
    grad: np.ndarray       # [W][N][3] grad ln psi
    lap: np.ndarray        # [W] sum_i lap_i psi / psi
    eloc: np.ndarray       # [W]
    O: np.ndarray | None   # [W][P] d ln psi / d theta


class LocalOperator:
    """act_on(batch) -> O psi / psi per walker: [W] (scalar) or [W][...] (vector)."""

    needs_O = False

    def act_on(self, batch: WalkerBatch) -> np.ndarray:
        raise NotImplementedError


class KineticEnergy(LocalOperator):
    """-1/2 lap psi / psi (operator.rs:103-125)."""

    def act_on(self, b):
        return -0.5 * b.lap


class IonicPotential(LocalOperator):
    """-sum_{I,i} Z_I / r_iI plus the constant ion-ion repulsion (operator.rs:15-62)."""

    def __init__(self, ion_positions, ion_charge):
        self.R = np.asarray(ion_positions, dtype=np.float64).reshape(-1, 3)
        self.Z = np.asarray(ion_charge, dtype=np.float64).reshape(-1)
        d = self.R[:, None, :] - self.R[None, :, :]
        r = np.linalg.norm(d, axis=-1)
        iu = np.triu_indices(self.R.shape[0], 1)
        self.repulsion = float(np.sum(np.outer(self.Z, self.Z)[iu] / r[iu]))

    def act_on(self, b):
        r = np.linalg.norm(b.pos[:, :, None, :] - self.R[None, None, :, :], axis=-1)  # [W][N][M]
        return -np.sum(self.Z[None, None, :] / r, axis=(1, 2)) + self.repulsion


class ElectronicPotential(LocalOperator):
    """sum_{i<j} 1 / r_ij (operator.rs:68-97)."""

    def act_on(self, b):
        N = b.pos.shape[1]
        if N < 2:
            return np.zeros(b.pos.shape[0])
        i, j = np.triu_indices(N, 1)
        return np.sum(1.0 / np.linalg.norm(b.pos[:, i] - b.pos[:, j], axis=-1), axis=1)


class ElectronicHamiltonian(LocalOperator):
    """Kinetic + ionic + electronic (operator.rs:150-184); equals the device's E_L."""

    def __init__(self, ion_positions, ion_charge):
        self.t, self.v_ion, self.v_ee = KineticEnergy(), IonicPotential(ion_positions, ion_charge), ElectronicPotential()

    @classmethod
    def from_system(cls, system):
        return cls(system.nuc_pos, system.nuc_z)

    def act_on(self, b):
        return self.t.act_on(b) + self.v_ion.act_on(b) + self.v_ee.act_on(b)


class WavefunctionValue(LocalOperator):
    """psi itself (act_on returns psi^2, divided by psi: src/vmc/src/operators.rs:16-24)."""

    def act_on(self, b):
        return b.sign * np.exp(b.lnpsi)


class ParameterGradient(LocalOperator):
    """d ln psi / d theta_k per walker (the corrected form of src/vmc/src/operators.rs:7-14)."""

    needs_O = True

    def act_on(self, b):
        return b.O


class HarmonicPotential(LocalOperator):
    """0.5 omega^2 |x|^2 summed over electrons (examples/custom_operator.rs:54-58)."""

    def __init__(self, frequency: float):
        self.frequency = frequency

    def act_on(self, b):
        return 0.5 * self.frequency ** 2 * np.sum(b.pos * b.pos, axis=(1, 2))


class HarmonicHamiltonian(LocalOperator):
    """KineticEnergy + HarmonicPotential (examples/custom_operator.rs:29-61)."""

    def __init__(self, frequency: float):
        self.t, self.v = KineticEnergy(), HarmonicPotential(frequency)

    def act_on(self, b):
        return self.t.act_on(b) + self.v.act_on(b)
