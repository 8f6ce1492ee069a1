"""Cell, k-mesh and the frozen plane-wave basis (host-side setup, NumPy).

Mirrors src/addft/geometry/cell.py:17-59, kmesh.py:19-59 and
basis.py:59-144 of the reference: the integer Miller sets and the FFT box are
fixed once on the reference geometry (they are index data, not part of the
hot path), physical G vectors are recomputed from the lattice on the GPU.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Cell:
    """Lattice rows a1, a2, a3 (Bohr) and fractional coordinates (nat, 3) (cell.py:17-25)."""
    lattice: np.ndarray
    frac: np.ndarray

    def __post_init__(self):
        object.__setattr__(self, "lattice", np.asarray(self.lattice, dtype=np.float64).reshape(3, 3))
        object.__setattr__(self, "frac", np.asarray(self.frac, dtype=np.float64).reshape(-1, 3))

    @property
    def natom(self) -> int:
        return int(self.frac.shape[0])


def reciprocal(lattice) -> np.ndarray:
    """B = 2 pi inv(L)^T, rows b1, b2, b3 (cell.py:28-30)."""
    return 2.0 * np.pi * np.linalg.inv(np.asarray(lattice, dtype=np.float64)).T


def volume(lattice) -> float:
    return abs(float(np.linalg.det(np.asarray(lattice, dtype=np.float64))))


def positions(cell: Cell) -> np.ndarray:
    return cell.frac @ cell.lattice


def with_frac(cell: Cell, frac) -> Cell:
    return Cell(lattice=cell.lattice, frac=frac)


def strained(cell: Cell, eps) -> Cell:
    """a_i' = a_i (I + eps), fractional coordinates fixed (cell.py:46-53)."""
    return Cell(lattice=cell.lattice @ (np.eye(3) + np.asarray(eps, dtype=np.float64)), frac=cell.frac)


def displacement(cell: Cell, delta) -> Cell:
    return with_frac(cell, cell.frac + np.asarray(delta) @ np.linalg.inv(cell.lattice))


@dataclass(frozen=True)
class KMesh:
    """Fractional k points with weights summing to 1 (kmesh.py:19-26)."""
    kfrac: np.ndarray
    weights: np.ndarray

    def cartesian(self, lattice) -> np.ndarray:
        return np.asarray(self.kfrac, dtype=np.float64) @ reciprocal(lattice)


def gamma() -> KMesh:
    return KMesh(kfrac=np.zeros((1, 3)), weights=np.ones(1))


def monkhorst_pack(n, shift=None) -> KMesh:
    """MP grid folded into [-0.5, 0.5) (kmesh.py:33-55)."""
    n = tuple(int(x) for x in n)
    shift = (0.0, 0.0, 0.0) if shift is None else tuple(float(x) for x in shift)
    pts = [((i + shift[0]) / n[0], (j + shift[1]) / n[1], (k + shift[2]) / n[2])
           for i in range(n[0]) for j in range(n[1]) for k in range(n[2])]
    frac = np.asarray(pts, dtype=np.float64)
    frac = np.where(frac >= 0.5, frac - 1.0, frac)
    return KMesh(kfrac=frac, weights=np.full(frac.shape[0], 1.0 / frac.shape[0]))


def check_weights(kmesh: KMesh) -> float:
    return float(abs(np.sum(kmesh.weights) - 1.0))


# ---------------------------------------------------------------------------
# basis (basis.py:59-144)
# ---------------------------------------------------------------------------

def shell_radius2(ecut: float) -> float:
    return 2.0 * float(ecut)


def is_smooth235(n: int) -> bool:
    if n < 1:
        return False
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


def smooth_up(n: int) -> int:
    while not is_smooth235(n):
        n += 1
    return n


def _nmax_on_axis(lattice, gcut2: float, kmax: float = 0.0):
    a_len = np.linalg.norm(np.asarray(lattice, dtype=np.float64), axis=1)
    m = np.ceil((np.sqrt(gcut2) + kmax) * a_len / (2.0 * np.pi)).astype(int)
    return int(m[0]), int(m[1]), int(m[2])


def build_miller(lattice, ecut: float, kpts=None) -> np.ndarray:
    """Union shell |k+G|^2 <= 2 ecut over k, ordered by |G|^2 then m lexicographic."""
    gcut2 = shell_radius2(ecut)
    lat = np.asarray(lattice, dtype=np.float64)
    bmat = 2.0 * np.pi * np.linalg.inv(lat).T
    ks = np.zeros((1, 3)) if kpts is None else np.asarray(kpts, dtype=np.float64)
    kmax = float(np.max(np.linalg.norm(ks, axis=1)))
    m1, m2, m3 = _nmax_on_axis(lat, gcut2, kmax)
    rng = np.stack(np.meshgrid(np.arange(-m1, m1 + 1), np.arange(-m2, m2 + 1),
                               np.arange(-m3, m3 + 1), indexing="ij"), axis=-1).reshape(-1, 3)
    bmat_inv = np.linalg.inv(bmat)
    keep = np.zeros(len(rng), dtype=bool)
    for k in ks:
        cart = (rng + k @ bmat_inv) @ bmat
        keep |= np.sum(cart ** 2, axis=1) <= gcut2 * (1.0 + 1e-12)
    miller = rng[keep]
    g2 = np.sum((miller @ bmat) ** 2, axis=1)
    order = np.lexsort((miller[:, 2], miller[:, 1], miller[:, 0], g2))
    return np.ascontiguousarray(miller[order].astype(np.int32))


def fft_shape(lattice, ecut: float, density_factor: float = 4.0) -> tuple:
    gcut2 = shell_radius2(ecut) * float(density_factor)
    return tuple(smooth_up(2 * m + 1) for m in _nmax_on_axis(lattice, gcut2))


@dataclass(frozen=True)
class Basis:
    """Frozen Miller sets (wavefunction and density shells) and the FFT box (basis.py:36-56)."""
    miller: np.ndarray
    ecut: float
    fft_shape: tuple
    miller_rho: np.ndarray

    @property
    def nG(self) -> int:
        return int(self.miller.shape[0])

    @property
    def nG_rho(self) -> int:
        return int(self.miller_rho.shape[0])

    @property
    def nfft(self) -> int:
        return int(np.prod(self.fft_shape))


def make_basis(lattice, ecut: float, density_factor: float = 4.0, kpts=None) -> Basis:
    ecut = float(ecut)
    return Basis(miller=build_miller(lattice, ecut, kpts=kpts), ecut=ecut,
                 fft_shape=fft_shape(lattice, ecut, density_factor),
                 miller_rho=build_miller(lattice, ecut * float(density_factor)))


def shell_margin(basis: Basis, lattice) -> float:
    g = basis.miller @ reciprocal(lattice)
    r2 = np.sum(g * g, axis=1)
    return float((shell_radius2(basis.ecut) - r2.max()) / shell_radius2(basis.ecut))
