"""Energies and their envelope gradients on the GPU.

Mirrors src/addft/observables/energy.py:22-169 (7 tagged terms, variational
energy, Mermin free energy) without dense matrices: every <psi|V|psi> is the
exact grid identity (Omega/N) sum_r v(r) rho_psi(r) (the same aliased DFT the
reference's vmat_from_real uses), and the band energy uses the matrix-free
H psi kernel.

The envelope gradient (api.py:106-113: psi and f frozen, rho = rho(geo, psi))
is assembled from hand-written gradient kernels:
  kinetic strain, Hartree and local terms from n(G) of rho(psi), the LDA
  volume term, the nonlocal position/strain terms, and Ewald.
"""

from __future__ import annotations

import numpy as np
import torch

from . import ops
from .geometry import Cell, volume
from .solver import density_of, effective_potential, wocc_of
from .system import GeometryCache, SCFState, Static, build_geometry_cache

ALL_TAGS = ("kinetic", "local", "hartree", "exchange", "correlation", "nonlocal", "ewald")


def _charges(static: Static):
    return np.full(static.natom, static.psp.zval, dtype=np.float64)


def _ewald(static: Static, geo: Cell, cache: GeometryCache):
    return ops.ewald(geo.lattice, cache.pos, _charges(static), eta=static.eta_ewald, nmax=8)


def _band_sum(static, psi, occ, x):
    """sum_k,b w_k f g_s Re <psi|x>  (x has psi's shape)."""
    w = wocc_of(static, occ)
    return torch.sum(w * torch.sum((psi.conj() * x).real, dim=-1))


def energy_terms(geo: Cell, static: Static, state: SCFState, active=ALL_TAGS, cache: GeometryCache = None):
    """dict[tag] -> float (Ha) (energy.py:36-71)."""
    cache = cache or build_geometry_cache(geo, static)
    dev = static.device()
    scale = cache.omega / static.basis.nfft
    out = {}
    rho_psi = None
    if "kinetic" in active:
        p2 = torch.abs(state.psi) ** 2
        out["kinetic"] = torch.sum(wocc_of(static, state.occ)[:, :, None] * p2 * cache.kin[:, None, :])
    if "local" in active:
        rho_psi = density_of(static, cache, state.psi, state.occ)
        out["local"] = scale * torch.sum(cache.v_loc_r * rho_psi)
    if "hartree" in active:
        out["hartree"] = ops.hartree(dev.wfc, cache.bvec, cache.omega, state.rho_r, want_potential=False)[1][0]
    if "exchange" in active or "correlation" in active:
        _, _, sums = ops.xc_lda(state.rho_r, want_vxc=False)
        if "exchange" in active:
            out["exchange"] = scale * sums[0]
        if "correlation" in active:
            out["correlation"] = scale * sums[1]
    if "nonlocal" in active:
        b = ops.becp(cache.proj, state.psi)
        out["nonlocal"] = ops.nonlocal_energy(b, cache.dion, wocc_of(static, state.occ))[0]
    if "ewald" in active:
        out["ewald"] = _ewald(static, geo, cache)[0]
    return {k: float(v) for k, v in out.items()}


def total_energy(geo, static, state, active=ALL_TAGS):
    return float(sum(energy_terms(geo, static, state, active).values()))


def energy_variational(geo: Cell, static: Static, state: SCFState, cache: GeometryCache = None):
    """E = sum f<psi|H[rho]|psi> - E_H + E_xc - <psi|V_xc|psi> + E_II (energy.py:134-153)."""
    cache = cache or build_geometry_cache(geo, static)
    scale = cache.omega / static.basis.nfft
    rho_psi = density_of(static, cache, state.psi, state.occ)
    v_eff, parts = effective_potential(static, cache, state.rho_r, rho_dc=rho_psi)
    hp = ops.hpsi(static.device().wfc, state.psi, cache.kin, v_eff, cache.proj, cache.dion)
    e_band = _band_sum(static, state.psi, state.occ, hp)
    sums = parts["xc_sums"]
    e_xc = scale * (sums[0] + sums[1])
    e_dc = scale * sums[2]
    e_ii = _ewald(static, geo, cache)[0]
    return float(e_band - parts["e_h"][0] + e_xc - e_dc + e_ii)


def entropy(occ: torch.Tensor, kweights: torch.Tensor) -> torch.Tensor:
    """S = -sum w [f ln f + (1-f) ln(1-f)] (occupation.py:68-72)."""
    f = torch.clamp(occ, 1e-14, 1.0 - 1e-14)
    s = -(f * torch.log(f) + (1.0 - f) * torch.log(1.0 - f))
    return torch.sum(kweights[:, None] * s)


def mermin_free_energy(geo: Cell, static: Static, state: SCFState, cache: GeometryCache = None):
    """F = E_var - sigma g_s S (energy.py:156-169)."""
    s = float(entropy(state.occ, static.kweights_t()))
    return energy_variational(geo, static, state, cache) - static.sigma * static.spin_degeneracy * s


def envelope_gradients(geo: Cell, static: Static, state: SCFState, cache: GeometryCache = None,
                       precision: str = "fp64"):
    """(dF/dR (nat, 3), dF/deps (3, 3)) with psi, f frozen and rho = rho(geo, psi).

    ``precision="fp32"`` runs the nonlocal contractions (the only part that
    scales with nb * nproj * nG) in FP32; every sum is accumulated in FP64.
    """
    cache = cache or build_geometry_cache(geo, static)
    dev = static.device()
    nat = static.natom
    scale = cache.omega / static.basis.nfft
    wocc = wocc_of(static, state.occ)
    rho = density_of(static, cache, state.psi, state.occ)
    deps = ops.kinetic_stress(dev.wfc, cache.bvec, static.kpts, state.psi, wocc).reshape(3, 3)
    dg = ops.density_gradients(dev.wfc, dev.rho, cache.bvec, cache.omega, cache.pos, static.psp, rho)
    dR = dg[5:5 + 3 * nat].reshape(nat, 3).clone()
    deps = deps + dg[5 + 3 * nat:5 + 3 * nat + 9].reshape(3, 3) + dg[5 + 3 * nat + 9:].reshape(3, 3)
    _, _, sums = ops.xc_lda(rho, want_vxc=False)
    deps = deps + (scale * (sums[0] + sums[1] - sums[2])) * torch.eye(3, dtype=torch.float64, device="cuda")
    psi = state.psi.to(torch.complex64) if precision == "fp32" else state.psi
    nl = ops.nonlocal_gradients(dev.wfc, cache.bvec, cache.omega, static.kpts, cache.pos, static.psp, psi, wocc,
                                cache.dion)
    dR = dR + nl[1:1 + 3 * nat].reshape(nat, 3)
    deps = deps + nl[1 + 3 * nat:].reshape(3, 3)
    ew = _ewald(static, geo, cache)
    dR = dR + ew[1:1 + 3 * nat].reshape(nat, 3)
    deps = deps + ew[1 + 3 * nat:].reshape(3, 3)
    return dR.cpu().numpy(), deps.cpu().numpy()


def forces_from_dR(dR) -> np.ndarray:
    """F = -dE/dR (implicit.py:95-101)."""
    return -np.asarray(dR)


def stress_from_deps(omega: float, deps) -> np.ndarray:
    """sigma = -(1/Omega) sym(dE/deps) (api.py:145-146, implicit.py:104-110)."""
    g = np.asarray(deps)
    return -(0.5 * (g + g.T)) / omega


# ---------------------------------------------------------------------------
# constraint observables (observables/constraint.py:26-57)
# ---------------------------------------------------------------------------

def delta_q(geo: Cell, static: Static, state: SCFState, weight) -> float:
    """C = int w(r) n(r) dr = (Omega/N) sum_j w_j n_j (constraint.py:26-33)."""
    w = torch.as_tensor(np.asarray(weight, dtype=np.float64), device="cuda")
    return float(volume(geo.lattice) / static.basis.nfft * torch.dot(w, state.rho_r))


def delta_q_grad(geo: Cell, static: Static, state: SCFState, weight, cache=None):
    """dC/dgeo through the fixed-point adjoint (constraint.py:36-44): C is not
    stationary in n, so (I - dF/dn)^T lambda = dC/dn is solved matrix-free.
    Returns (Cell of gradients, diagnostics)."""
    from .response import implicit_grad
    w = torch.as_tensor(np.asarray(weight, dtype=np.float64), device="cuda")
    g_n = (volume(geo.lattice) / static.basis.nfft) * w
    q = delta_q(geo, static, state, weight)
    return implicit_grad(geo, static, state, g_n, dL_deps=q * np.eye(3), cache=cache, return_diagnostics=True)


def make_gaussian_weight(basis, center, sigma: float = 0.8, lattice=None) -> np.ndarray:
    """Normalised Gaussian weight on the FFT grid, (Omega/N) sum w ~ 1 (constraint.py:47-57)."""
    shape = tuple(basis.fft_shape)
    idx = np.stack(np.meshgrid(*(np.arange(n) for n in shape), indexing="ij"), -1).reshape(-1, 3)
    r = (idx / np.asarray(shape, dtype=np.float64)) @ np.asarray(lattice, dtype=np.float64)
    w = np.exp(-0.5 * np.sum((r - np.asarray(center)) ** 2, axis=-1) / sigma ** 2)
    return w / np.sum(w) * basis.nfft
