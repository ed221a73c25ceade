"""Generates tests/golden/trial_functions.npz: golden ln psi, grad ln psi,
lap psi / psi and E_L of the reference's own trial functions at seeded
positions, from their closed forms written out here in numpy.

The reference (Jvanrhijn/mole, Rust) cannot be built here, so these vectors
are the independent pin of the CPU oracle and the GPU path: each closed form
below is derived by hand from the trial function and Hamiltonian the
reference's examples and tests define, not from the oracle's code.

  H-sto       psi = exp(-a r), H atom                 examples/dmc.rs:94-149
  He-product  psi = exp(-a (r1 + r2)), He             tests/helium_lcao.rs:22-87
  He-pade     He product x exp(r12 / (2 (1 + b r12))) (the helium singlet VMC workload)
  H2+product  psi = exp(-a (rA + rB)), one electron   tests/hydrogen_molecular_ion_lcao.rs:20-92
  SHO         psi = exp(-(r/a)^2), harmonic well      examples/custom_operator.rs:29-98
  H2-pade     sigma(r1) sigma(r2) exp(u(r12)),        examples/hydrogen_molecule.rs:64-168 (with
              sigma = exp(-a rA) + exp(-a rB)          the Pade e-e factor of theory/jastrow.tex:15-29)

Run:  python tests/golden/make_golden.py   (deterministic; rewrites the .npz)
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "trial_functions.npz")
N_CONF = 64

# name -> parameters (the test side maps each name to the same system)
PARAMS = {
    "H-sto": {"alpha": 0.8},
    "He-product": {"alpha": 1.69},
    "He-pade": {"alpha": 1.6875, "beta": 0.3},
    "H2+product": {"alpha": 1.0, "separation": 2.5},
    "SHO": {"a": 1.3, "omega": 0.9},
    "H2-pade": {"alpha": 1.0, "b": 0.5, "half_bond": 0.7},
}


def _norm(v):
    return np.linalg.norm(v, axis=-1)


def h_sto(pos, alpha):
    x = pos[:, 0]
    r = _norm(x)
    lnpsi = -alpha * r
    grad = (-alpha * x / r[:, None])[:, None, :]
    lap = alpha * alpha - 2.0 * alpha / r
    eloc = -0.5 * lap - 1.0 / r
    return lnpsi, grad, lap, eloc


def pade(r, cusp, beta):
    q = 1.0 / (1.0 + beta * r)
    return cusp * r * q, cusp * q * q, -2.0 * cusp * beta * q ** 3


def he(pos, alpha, beta=None):
    x1, x2 = pos[:, 0], pos[:, 1]
    r1, r2 = _norm(x1), _norm(x2)
    d = x1 - x2
    r12 = _norm(d)
    lnpsi = -alpha * (r1 + r2)
    g1 = -alpha * x1 / r1[:, None]
    g2 = -alpha * x2 / r2[:, None]
    l1 = -2.0 * alpha / r1
    l2 = -2.0 * alpha / r2
    if beta is not None:
        u, up, upp = pade(r12, 0.5, beta)
        lnpsi = lnpsi + u
        e = d / r12[:, None]
        g1 = g1 + up[:, None] * e
        g2 = g2 - up[:, None] * e
        l1 = l1 + upp + 2.0 * up / r12
        l2 = l2 + upp + 2.0 * up / r12
    lap = l1 + np.sum(g1 * g1, -1) + l2 + np.sum(g2 * g2, -1)
    eloc = -0.5 * lap - 2.0 / r1 - 2.0 / r2 + 1.0 / r12
    return lnpsi, np.stack([g1, g2], 1), lap, eloc


def h2_ion(pos, alpha, separation):
    h = 0.5 * separation
    x = pos[:, 0]
    dA, dB = x - np.array([h, 0, 0]), x - np.array([-h, 0, 0])
    rA, rB = _norm(dA), _norm(dB)
    lnpsi = -alpha * (rA + rB)
    g = -alpha * (dA / rA[:, None] + dB / rB[:, None])
    l = -2.0 * alpha * (1.0 / rA + 1.0 / rB)
    lap = l + np.sum(g * g, -1)
    eloc = -0.5 * lap - 1.0 / rA - 1.0 / rB + 1.0 / separation
    return lnpsi, g[:, None, :], lap, eloc


def sho(pos, a, omega):
    x = pos[:, 0]
    r2 = np.sum(x * x, -1)
    lnpsi = -r2 / (a * a)
    g = -2.0 * x / (a * a)
    lap = -6.0 / (a * a) + np.sum(g * g, -1)
    eloc = -0.5 * lap + 0.5 * omega * omega * r2
    return lnpsi, g[:, None, :], lap, eloc


def h2(pos, alpha, b, half_bond):
    A, B = np.array([0, 0, -half_bond]), np.array([0, 0, half_bond])
    grads, laps, lns, pot = [], [], [], 0.0
    for i in range(2):
        x = pos[:, i]
        dA, dB = x - A, x - B
        rA, rB = _norm(dA), _norm(dB)
        eA, eB = np.exp(-alpha * rA), np.exp(-alpha * rB)
        sig = eA + eB
        gs = -alpha * (eA[:, None] * dA / rA[:, None] + eB[:, None] * dB / rB[:, None])
        ls = eA * (alpha * alpha - 2.0 * alpha / rA) + eB * (alpha * alpha - 2.0 * alpha / rB)
        g = gs / sig[:, None]
        lns.append(np.log(sig))
        grads.append(g)
        laps.append(ls / sig - np.sum(g * g, -1))  # lap ln sigma
        pot = pot - 1.0 / rA - 1.0 / rB
    d = pos[:, 0] - pos[:, 1]
    r12 = _norm(d)
    u, up, upp = pade(r12, 0.5, b)
    e = d / r12[:, None]
    g1 = grads[0] + up[:, None] * e
    g2 = grads[1] - up[:, None] * e
    l1 = laps[0] + upp + 2.0 * up / r12
    l2 = laps[1] + upp + 2.0 * up / r12
    lnpsi = lns[0] + lns[1] + u
    lap = l1 + np.sum(g1 * g1, -1) + l2 + np.sum(g2 * g2, -1)
    eloc = -0.5 * lap + pot + 1.0 / r12 + 1.0 / (2.0 * half_bond)
    return lnpsi, np.stack([g1, g2], 1), lap, eloc


FUNCS = {
    "H-sto": (1, lambda p: h_sto(p, **PARAMS["H-sto"])),
    "He-product": (2, lambda p: he(p, PARAMS["He-product"]["alpha"])),
    "He-pade": (2, lambda p: he(p, **PARAMS["He-pade"])),
    "H2+product": (1, lambda p: h2_ion(p, **PARAMS["H2+product"])),
    "SHO": (1, lambda p: sho(p, **PARAMS["SHO"])),
    "H2-pade": (2, lambda p: h2(p, **PARAMS["H2-pade"])),
}


def generate() -> dict:
    out = {}
    for k, (name, (n_elec, f)) in enumerate(FUNCS.items()):
        pos = np.random.default_rng(1000 + k).normal(0.0, 1.3, size=(N_CONF, n_elec, 3))
        lnpsi, grad, lap, eloc = f(pos)
        out[f"{name}/pos"] = pos
        out[f"{name}/lnpsi"] = lnpsi
        out[f"{name}/grad"] = grad
        out[f"{name}/lap"] = lap
        out[f"{name}/eloc"] = eloc
    return out


if __name__ == "__main__":
    np.savez_compressed(OUT, **generate())
    print(f"wrote {OUT}")
