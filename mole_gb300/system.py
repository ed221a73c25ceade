"""Wavefunction/Hamiltonian descriptors for the mole walker hot path.

The reference (Jvanrhijn/mole) lets a user implement the ``Function`` /
``Differentiate`` / ``WaveFunction`` / ``Optimize`` traits for any psi
(``src/wavefunction_traits/src/lib.rs:7-24``, ``src/optimize/src/traits.rs:8-16``).
A per-walker trait object cannot cross into a GPU kernel, so this package
chooses the wavefunction *family* by descriptor: a Slater determinant per spin
block over Slater/Gaussian basis functions on the nuclei, times a Jastrow
factor (Pade e-e of ``theory/jastrow.tex:15-29``, a Pade e-n term and an
optional pairwise neural network). The reference's own example and test
trial functions are members of this family (see the builders below), which is
how they are used as known-answer checks.

Parameter vector layout (``System.params()``), the order of O_k:
``[orbital exponents] [e-e b, e-e polynomial b_3..] [e-n a] [neural weights]``,
each group present only when its term is switched on.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field

import numpy as np

STO_1S, STO_2S, STO_2PX, STO_2PY, STO_2PZ, GTO_1S = range(6)
POT_COULOMB, POT_HARMONIC = 0, 1
MOVE_BOX, MOVE_GAUSS, MOVE_DIFFUSE = 0, 1, 2

MAX_NUC = 8
MAX_BASIS = 32
MAX_SPIN = 5
MAX_POLY = 4
NN_H = 64
NN_IN = 4
NN_NET_P = NN_H * NN_IN + NN_H + NN_H * NN_H + NN_H + NN_H + 1  # 4545
NN_P = 2 * NN_NET_P  # e-e net + e-n net = 9090


def _arr(x, dtype=np.float64):
    return np.ascontiguousarray(np.asarray(x, dtype=dtype))


@dataclass
class System:
    nuc_pos: np.ndarray
    nuc_z: np.ndarray
    n_up: int
    n_dn: int
    basis_center: np.ndarray
    basis_kind: np.ndarray
    basis_exp: np.ndarray
    exponents: np.ndarray
    coef_up: np.ndarray
    coef_dn: np.ndarray
    ee_on: bool = False
    ee_b: float = 0.0
    ee_kappa: float = 0.0
    ee_poly: np.ndarray = field(default_factory=lambda: np.zeros(0))
    cusp_anti: float = 0.5
    cusp_para: float = 0.25
    en_on: bool = False
    en_a: float = 0.0
    en_coef: np.ndarray | None = None
    nn_on: bool = False
    nn_weights: np.ndarray | None = None
    pot_kind: int = POT_COULOMB
    omega: float = 0.0
    name: str = ""

    def __post_init__(self):
        self.nuc_pos = _arr(self.nuc_pos).reshape(-1, 3)
        self.nuc_z = _arr(self.nuc_z, np.int32).reshape(-1)
        self.basis_center = _arr(self.basis_center, np.int32).reshape(-1)
        self.basis_kind = _arr(self.basis_kind, np.int32).reshape(-1)
        self.basis_exp = _arr(self.basis_exp, np.int32).reshape(-1)
        self.exponents = _arr(self.exponents).reshape(-1)
        nb = self.basis_center.size
        self.coef_up = _arr(self.coef_up).reshape(self.n_up, nb)
        self.coef_dn = _arr(self.coef_dn).reshape(self.n_dn, nb)
        self.ee_poly = _arr(self.ee_poly).reshape(-1)
        if self.en_coef is None:
            self.en_coef = np.zeros(self.n_nuc)
        self.en_coef = _arr(self.en_coef).reshape(-1)
        if self.nn_on and self.nn_weights is None:
            self.nn_weights = np.zeros(NN_P)
        if self.nn_weights is not None:
            self.nn_weights = _arr(self.nn_weights).reshape(-1)
        self.validate()

    # ------------------------------------------------------------------ sizes
    @property
    def n_nuc(self) -> int:
        return int(self.nuc_pos.shape[0])

    @property
    def n_elec(self) -> int:
        return self.n_up + self.n_dn

    @property
    def n_basis(self) -> int:
        return int(self.basis_center.size)

    @property
    def n_exp(self) -> int:
        return int(self.exponents.size)

    @property
    def n_params(self) -> int:
        return (self.n_exp + (1 + self.ee_poly.size if self.ee_on else 0) + (1 if self.en_on else 0)
                + (NN_P if self.nn_on else 0))

    def validate(self) -> None:
        if not (1 <= self.n_nuc <= MAX_NUC):
            raise ValueError(f"1..{MAX_NUC} nuclei supported, got {self.n_nuc}")
        if not (0 <= self.n_dn <= self.n_up <= MAX_SPIN) or self.n_up < 1:
            raise ValueError("need 1 <= n_dn... : 0 <= n_dn <= n_up <= 5 and n_up >= 1")
        if not (1 <= self.n_basis <= MAX_BASIS):
            raise ValueError(f"1..{MAX_BASIS} basis functions supported")
        if self.basis_center.min() < 0 or self.basis_center.max() >= self.n_nuc:
            raise ValueError("basis centre index out of range")
        if self.basis_exp.min() < 0 or self.basis_exp.max() >= self.n_exp:
            raise ValueError("basis exponent index out of range")
        if self.basis_kind.min() < 0 or self.basis_kind.max() > GTO_1S:
            raise ValueError("unknown basis kind")
        if self.ee_poly.size > MAX_POLY:
            raise ValueError(f"at most {MAX_POLY} polynomial Jastrow terms")

    # ------------------------------------------------------------- parameters
    def params(self) -> np.ndarray:
        parts = [self.exponents]
        if self.ee_on:
            parts += [np.array([self.ee_b]), self.ee_poly]
        if self.en_on:
            parts.append(np.array([self.en_a]))
        if self.nn_on:
            parts.append(self.nn_weights)
        return np.ascontiguousarray(np.concatenate(parts))

    def with_params(self, theta) -> "System":
        theta = np.asarray(theta, dtype=np.float64)
        if theta.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {theta.size}")
        o = 0
        kw = {}
        kw["exponents"] = theta[o:o + self.n_exp].copy(); o += self.n_exp
        if self.ee_on:
            kw["ee_b"] = float(theta[o]); o += 1
            kw["ee_poly"] = theta[o:o + self.ee_poly.size].copy(); o += self.ee_poly.size
        if self.en_on:
            kw["en_a"] = float(theta[o]); o += 1
        if self.nn_on:
            kw["nn_weights"] = theta[o:o + NN_P].copy(); o += NN_P
        return dataclasses.replace(self, **kw)

    def nuclear_repulsion(self) -> float:
        """Constant n-n term added by IonicPotential::new (src/operator/src/operator.rs:42-49)."""
        v = 0.0
        for i in range(self.n_nuc):
            for j in range(i + 1, self.n_nuc):
                v += float(self.nuc_z[i] * self.nuc_z[j]) / float(np.linalg.norm(self.nuc_pos[i] - self.nuc_pos[j]))
        return v


# ---------------------------------------------------------------- builders

def helium(alpha: float = 1.6875, beta: float = 0.3) -> System:
    """He singlet, psi = exp(-alpha (r1 + r2)) exp(r12 / (2 (1 + beta r12)))."""
    return System(nuc_pos=[[0, 0, 0]], nuc_z=[2], n_up=1, n_dn=1, basis_center=[0], basis_kind=[STO_1S],
                  basis_exp=[0], exponents=[alpha], coef_up=[[1.0]], coef_dn=[[1.0]], ee_on=True, ee_b=beta,
                  name="He")


def helium_product(alpha: float) -> System:
    """Jastrow-free He product exp(-alpha (r1 + r2)) of tests/helium_lcao.rs:48-87."""
    return System(nuc_pos=[[0, 0, 0]], nuc_z=[2], n_up=1, n_dn=1, basis_center=[0], basis_kind=[STO_1S],
                  basis_exp=[0], exponents=[alpha], coef_up=[[1.0]], coef_dn=[[1.0]], name="He-product")


def h2(alpha: float = 1.0, b: float = 0.5, half_bond: float = 0.7) -> System:
    """H2, psi = sigma(r1) sigma(r2) Pade(r12), sigma = exp(-alpha r_A) + exp(-alpha r_B),
    nuclei at z = +-half_bond; parameters (alpha, b)."""
    return System(nuc_pos=[[0, 0, -half_bond], [0, 0, half_bond]], nuc_z=[1, 1], n_up=1, n_dn=1,
                  basis_center=[0, 1], basis_kind=[STO_1S, STO_1S], basis_exp=[0, 0], exponents=[alpha],
                  coef_up=[[1.0, 1.0]], coef_dn=[[1.0, 1.0]], ee_on=True, ee_b=b, name="H2")


def h2_ion_product(alpha: float = 1.0, separation: float = 2.5) -> System:
    """One electron, psi = phi(x - R/2) phi(x + R/2) with phi = exp(-alpha r)
    (tests/hydrogen_molecular_ion_lcao.rs:66-92): a 1s determinant on the
    nucleus at +R/2 times a linear e-n Jastrow -alpha r on the one at -R/2."""
    h = 0.5 * separation
    return System(nuc_pos=[[h, 0, 0], [-h, 0, 0]], nuc_z=[1, 1], n_up=1, n_dn=0, basis_center=[0],
                  basis_kind=[STO_1S], basis_exp=[0], exponents=[alpha], coef_up=[[1.0]], coef_dn=np.zeros((0, 1)),
                  en_on=True, en_a=0.0, en_coef=[0.0, -alpha], name="H2+-product")


def sho_gaussian(a: float, omega: float = 1.0) -> System:
    """3-D harmonic well with psi = exp(-(|x|/a)^2) (examples/custom_operator.rs:288-322)."""
    return System(nuc_pos=[[0, 0, 0]], nuc_z=[0], n_up=1, n_dn=0, basis_center=[0], basis_kind=[GTO_1S],
                  basis_exp=[0], exponents=[1.0 / (a * a)], coef_up=[[1.0]], coef_dn=np.zeros((0, 1)),
                  pot_kind=POT_HARMONIC, omega=omega, name="SHO")


def hydrogen_gaussian(a: float = 1.0) -> System:
    """H atom with the Gaussian trial function of examples/dmc.rs:366-430."""
    return System(nuc_pos=[[0, 0, 0]], nuc_z=[1], n_up=1, n_dn=0, basis_center=[0], basis_kind=[GTO_1S],
                  basis_exp=[0], exponents=[1.0 / (a * a)], coef_up=[[1.0]], coef_dn=np.zeros((0, 1)),
                  name="H-gaussian")


def hydrogen_sto(alpha: float = 1.0) -> System:
    """H atom with the STO trial function exp(-alpha r) of examples/dmc.rs:94-149."""
    return System(nuc_pos=[[0, 0, 0]], nuc_z=[1], n_up=1, n_dn=0, basis_center=[0], basis_kind=[STO_1S],
                  basis_exp=[0], exponents=[alpha], coef_up=[[1.0]], coef_dn=np.zeros((0, 1)), name="H-sto")


_SHELL = [STO_1S, STO_2S, STO_2PX, STO_2PY, STO_2PZ]


def random_atom(rng: np.random.Generator, z_range=(2, 10), n_range=(2, 10)) -> System:
    """One member of the ragged batch: Z in U{2..10}, N in U{2..10} electrons,
    N_up = ceil(N/2); 1s/2s/2p STOs with exponents U[0.5, Z]; Pade e-e
    b in U[0.2, 1] and e-n a in U[0.5, 2]."""
    Z = int(rng.integers(z_range[0], z_range[1] + 1))
    N = int(rng.integers(n_range[0], n_range[1] + 1))
    nu, nd = (N + 1) // 2, N // 2
    ex = rng.uniform(0.5, float(Z), size=5)
    eye = np.eye(5)
    return System(nuc_pos=[[0, 0, 0]], nuc_z=[Z], n_up=nu, n_dn=nd, basis_center=[0] * 5, basis_kind=_SHELL,
                  basis_exp=list(range(5)), exponents=ex, coef_up=eye[:nu], coef_dn=eye[:nd], ee_on=True,
                  ee_b=float(rng.uniform(0.2, 1.0)), en_on=True, en_a=float(rng.uniform(0.5, 2.0)),
                  en_coef=[-0.25 * Z], name=f"Z{Z}N{N}")


def nn_init(rng: np.random.Generator, std: float = 0.01) -> np.ndarray:
    """Gaussian N(0, std^2) initial weights for both pair networks."""
    return rng.normal(0.0, std, size=NN_P)


def lih(neural: bool = True, rng: np.random.Generator | None = None, b: float = 1.0) -> System:
    """LiH, Li (Z=3) at the origin and H (Z=1) at z = 3.015 bohr, 2 up / 2 down,
    minimal STO determinant (Li 1s, Li 2s, H 1s) with a Pade e-e Jastrow and,
    if ``neural``, the pairwise-MLP Jastrow on top."""
    rng = rng or np.random.default_rng(0x5EED + 4)
    # basis: Li 1s (zeta 2.69), Li 2s (0.65), H 1s (1.0), Li 2pz (0.65)
    coef = np.array([[1.0, 0.0, 0.0, 0.0], [0.0, 0.55, 0.55, 0.3]])
    return System(nuc_pos=[[0, 0, 0], [0, 0, 3.015]], nuc_z=[3, 1], n_up=2, n_dn=2,
                  basis_center=[0, 0, 1, 0], basis_kind=[STO_1S, STO_2S, STO_1S, STO_2PZ],
                  basis_exp=[0, 1, 2, 1], exponents=[2.69, 0.65, 1.0], coef_up=coef, coef_dn=coef, ee_on=True,
                  ee_b=b, nn_on=neural, nn_weights=nn_init(rng) if neural else None, name="LiH")


def beryllium(neural: bool = False, rng: np.random.Generator | None = None, b: float = 1.0,
              cusp: bool = False) -> System:
    """Be (Z=4), 2 up / 2 down, 1s/2s STO determinant with a Pade e-e Jastrow
    and optionally the pairwise-MLP Jastrow. With ``cusp`` a Pade e-n term
    A r / (1 + a r), A = -(Z - zeta_1s), restores the nuclear cusp the 1s
    exponent alone misses (the DMC guide's Pade fallback)."""
    rng = rng or np.random.default_rng(0x5EED + 5)
    coef = np.eye(2)
    z1s = 3.7
    return System(nuc_pos=[[0, 0, 0]], nuc_z=[4], n_up=2, n_dn=2, basis_center=[0, 0],
                  basis_kind=[STO_1S, STO_2S], basis_exp=[0, 1], exponents=[z1s, 0.975], coef_up=coef,
                  coef_dn=coef, ee_on=True, ee_b=b, en_on=cusp, en_a=1.0 if cusp else 0.0,
                  en_coef=[-(4.0 - z1s)] if cusp else None, nn_on=neural,
                  nn_weights=nn_init(rng) if neural else None, name="Be")
