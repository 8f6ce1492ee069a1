"""Static discretisation data, SCF state and the per-geometry device cache.

Mirrors src/addft/system.py:24-69 and solver/geometry_cache.py:26-39.  The
only differentiable input is the ``Cell``; ``Static`` holds the frozen
integer data (Miller sets, box), the k mesh, the pseudopotential and the
electron count.  ``Static.device()`` owns the GPU plans of the two shells.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch

from . import ops
from .geometry import Basis, Cell, KMesh, make_basis, positions, reciprocal, volume
from .psp import Pseudo, dion_full


class DeviceStatic:
    """GPU resources that depend only on the frozen basis: plans of both shells
    (and, on first use, a plan of the whole box for the Kerker preconditioner)."""

    def __init__(self, basis: Basis):
        ops.require_cuda()
        self.basis = basis
        self.wfc = ops.Plan(basis.fft_shape, basis.miller)
        self.rho = ops.Plan(basis.fft_shape, basis.miller_rho)
        self._full = None

    @property
    def full(self):
        """Every box point, Miller indices folded to [-n/2, n/2) as the reference's q2_grid (scf.py:202-212)."""
        if self._full is None:
            n1, n2, n3 = self.basis.fft_shape
            ax = [np.where(np.arange(n) < n // 2, np.arange(n), np.arange(n) - n) for n in (n1, n2, n3)]
            m = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3).astype(np.int32)
            self._full = ops.Plan(self.basis.fft_shape, m)
        return self._full


@dataclass
class Static:
    basis: Basis
    kpts: np.ndarray          # (nk, 3) Cartesian, fixed at setup (system.py:62)
    kweights: np.ndarray      # (nk,), sum 1
    psp: Pseudo
    natom: int
    nband: int
    spin_degeneracy: float
    sigma: float
    nelec: float
    eta_ewald: float
    _dev: Optional[DeviceStatic] = field(default=None, repr=False, compare=False)

    @property
    def nk(self) -> int:
        return int(self.kpts.shape[0])

    def device(self) -> DeviceStatic:
        if self._dev is None:
            self._dev = DeviceStatic(self.basis)
        return self._dev

    def kweights_t(self) -> torch.Tensor:
        return torch.as_tensor(self.kweights, dtype=torch.float64, device="cuda")


@dataclass
class SCFState:
    """psi (nk, nband, nG) complex128 on the device, eig/occ (nk, nband), mu, rho_r (N,)."""
    psi: torch.Tensor
    eig: torch.Tensor
    occ: torch.Tensor
    mu: torch.Tensor
    rho_r: torch.Tensor
    n_iter: int
    residual: float

    def _replace(self, **kw) -> "SCFState":
        d = dict(self.__dict__)
        d.update(kw)
        return SCFState(**d)


def make_static(cell: Cell, psp: Pseudo, kmesh: KMesh, ecut: float, nband: int, sigma: float = 0.01,
                density_factor: float = 4.0, eta_ewald: float = 0.9) -> Static:
    """system.py:47-69 (multi-species is rejected; sigma default 0.01 here, 0.05 via setup)."""
    if psp.nspec != 1:
        raise NotImplementedError("multiple species are rejected explicitly (system.py:53-54)")
    if psp.nlcc:
        raise NotImplementedError("NLCC pseudopotentials are rejected (psp.py:169-172)")
    kpts = kmesh.cartesian(cell.lattice)
    basis = make_basis(cell.lattice, ecut, density_factor, kpts=kpts)
    return Static(basis=basis, kpts=np.asarray(kpts, dtype=np.float64),
                  kweights=np.asarray(kmesh.weights, dtype=np.float64), psp=psp, natom=cell.natom,
                  nband=int(nband), spin_degeneracy=2.0, sigma=float(sigma),
                  nelec=float(psp.zval * cell.natom), eta_ewald=float(eta_ewald))


@dataclass
class GeometryCache:
    """Per-geometry device tables (geometry_cache.py:26-39) in both precisions on demand."""
    v_loc_r: torch.Tensor          # (N,) f64
    proj: torch.Tensor             # (nk, nat*nh, nG) complex128
    dion: torch.Tensor             # (P, P) f64
    kin: torch.Tensor              # (nk, nG) f64
    bvec: np.ndarray
    omega: float
    pos: np.ndarray
    _f32: Optional[tuple] = field(default=None, repr=False)

    def f32(self):
        if self._f32 is None:
            self._f32 = (self.proj.to(torch.complex64), self.dion.to(torch.float32), self.kin.to(torch.float32))
        return self._f32


def build_geometry_cache(geo: Cell, static: Static) -> GeometryCache:
    dev = static.device()
    bvec = reciprocal(geo.lattice)
    omega = volume(geo.lattice)
    pos = positions(geo)
    v_loc = ops.local_potential(dev.rho, bvec, omega, pos, static.psp)
    proj = ops.projectors(dev.wfc, bvec, omega, static.kpts, pos, static.psp, dtype=torch.complex128)
    dion = torch.as_tensor(dion_full(static.psp, static.natom), dtype=torch.float64, device="cuda")
    kin = ops.kinetic(dev.wfc, bvec, static.kpts, dtype=torch.float64)
    return GeometryCache(v_loc_r=v_loc, proj=proj, dion=dion, kin=kin, bvec=bvec, omega=omega, pos=pos)
