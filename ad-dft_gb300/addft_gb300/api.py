"""Public API, unchanged from the reference (src/addft/api.py:30-152).

``setup`` builds the static discretisation; ``scf``/``energy``/
``energy_explicit`` run the GPU SCF; ``energy_and_forces`` and ``stress``
return the envelope derivatives of the Mermin free energy computed by the
GB300 gradient kernels; ``make_energy`` returns a differentiable scalar
function of the ``Cell`` (a ``torch.autograd.Function`` whose backward is
the envelope gradient, or with mode="adjoint" the fixed-point adjoint -- the
analogue of the reference's ``jax.custom_vjp``).
"""

from __future__ import annotations

from typing import NamedTuple

import numpy as np
import torch

from . import observables as obs
from .geometry import Cell, KMesh, gamma, strained, volume
from .psp import Pseudo, synthetic
from .solver import solve_scf
from .system import SCFState, Static, build_geometry_cache, make_static


class System(NamedTuple):
    geo: Cell
    static: Static


def setup(lattice, frac, psp: Pseudo | None = None, ecut: float = 8.0, nband: int = 4,
          kmesh: KMesh | None = None, sigma: float = 0.05, density_factor: float = 4.0,
          eta_ewald: float = 0.9, spec_idx=None) -> System:
    """api.py:35-45."""
    geo = Cell(lattice=lattice, frac=frac)
    psp = synthetic() if psp is None else psp
    if spec_idx is not None and len(set(np.asarray(spec_idx).reshape(-1).tolist())) > 1:
        raise NotImplementedError("multiple species are rejected (system.py:53-54)")
    static = make_static(geo, psp, kmesh or gamma(), ecut, nband, sigma=sigma,
                         density_factor=density_factor, eta_ewald=eta_ewald)
    return System(geo=geo, static=static)


def scf(system: System, **kwargs) -> SCFState:
    return solve_scf(system.geo, system.static, **kwargs)


def energy(system: System, state: SCFState | None = None, **kwargs) -> float:
    """Mermin free energy F = E_var - sigma g_s S (api.py:58-61)."""
    state = scf(system, **kwargs) if state is None else state
    return obs.mermin_free_energy(system.geo, system.static, state)


def energy_explicit(system: System, state: SCFState | None = None) -> float:
    """Explicit 7-term functional (api.py:64-67)."""
    state = scf(system) if state is None else state
    return obs.total_energy(system.geo, system.static, state)


def _split_kwargs(kw):
    grad_precision = kw.pop("grad_precision", None)
    prec = kw.get("precision", "fp64")
    return kw, grad_precision or prec


class _EnergyFn(torch.autograd.Function):
    """F(lattice, frac) with the reference's two backward paths (api.py:94-118):
    mode "envelope" (psi, f frozen, rho = rho(geo, psi)) or "adjoint" (fixed-point
    implicit differentiation of F with psi, f frozen, implicit.py:32-87)."""

    @staticmethod
    def forward(ctx, lattice, frac, static, scf_kwargs, mode="envelope", adjoint_mode="matrix_free"):
        kw, gprec = _split_kwargs(dict(scf_kwargs))
        geo = Cell(lattice=lattice.detach().cpu().numpy(), frac=frac.detach().cpu().numpy())
        cache = build_geometry_cache(geo, static)
        state = solve_scf(geo, static, cache=cache, **kw)
        e = obs.mermin_free_energy(geo, static, state, cache)
        ctx.save = (geo, static, state, cache, gprec, mode, adjoint_mode)
        return torch.as_tensor(e, dtype=torch.float64)

    @staticmethod
    def backward(ctx, g):
        geo, static, state, cache, gprec, mode, adjoint_mode = ctx.save
        L = geo.lattice
        if mode == "envelope":
            dR, deps = obs.envelope_gradients(geo, static, state, cache, precision=gprec)
            d_frac = dR @ L.T                       # R = frac L
            d_lat = np.linalg.inv(L).T @ deps       # L' = L (I + eps) -> dE/deps = L^T dE/dL
        else:
            from .response import energy_implicit_grad
            grad = energy_implicit_grad(geo, static, state, cache=cache, mode=adjoint_mode)
            d_lat, d_frac = np.asarray(grad.lattice), np.asarray(grad.frac)
        gv = float(g)
        return (torch.as_tensor(gv * d_lat, dtype=torch.float64), torch.as_tensor(gv * d_frac, dtype=torch.float64),
                None, None, None, None)


def make_energy(static: Static, mode: str = "envelope", adjoint_mode: str = "matrix_free", **scf_kwargs):
    """Differentiable scalar F(geo) (api.py:70-119).

    Returns ``f`` with ``f(cell) -> float`` and ``f.value_and_grad(cell) ->
    (F, Cell(lattice=dF/dL, frac=dF/dfrac))``; ``f.torch(lattice_t, frac_t)``
    is the torch-differentiable form.  ``mode="envelope"`` (default, the
    production path) freezes psi and f and rebuilds rho from psi at the new
    geometry; ``mode="adjoint"`` routes the backward through the fixed-point
    adjoint like the reference (api.py:114-116), with ``adjoint_mode``
    "matrix_free" (BiCGSTAB) or "dense" (assembled Jacobian, small boxes).
    """
    if mode not in ("envelope", "adjoint"):
        raise ValueError(f"unknown mode {mode!r}: 'envelope' or 'adjoint'")
    if adjoint_mode not in ("matrix_free", "dense"):
        raise ValueError(f"unknown adjoint_mode {adjoint_mode!r}: 'matrix_free' or 'dense'")

    class EnergyFn:
        def __call__(self, geo: Cell) -> float:
            cache = build_geometry_cache(geo, static)
            kw, _ = _split_kwargs(dict(scf_kwargs))
            st = solve_scf(geo, static, cache=cache, **kw)
            return obs.mermin_free_energy(geo, static, st, cache)

        def torch(self, lattice_t, frac_t):
            return _EnergyFn.apply(lattice_t, frac_t, static, scf_kwargs, mode, adjoint_mode)

        def value_and_grad(self, geo: Cell):
            lat = torch.tensor(geo.lattice, dtype=torch.float64, requires_grad=True)
            fr = torch.tensor(geo.frac, dtype=torch.float64, requires_grad=True)
            e = self.torch(lat, fr)
            e.backward()
            return float(e.detach()), Cell(lattice=lat.grad.numpy(), frac=fr.grad.numpy())

    return EnergyFn()


def energy_and_forces(system: System, **scf_kwargs):
    """(F, forces (nat, 3) Ha/Bohr) from one SCF and one envelope gradient (api.py:122-128)."""
    kw, gprec = _split_kwargs(dict(scf_kwargs))
    geo, static = system.geo, system.static
    cache = build_geometry_cache(geo, static)
    state = solve_scf(geo, static, cache=cache, **kw)
    e = obs.mermin_free_energy(geo, static, state, cache)
    dR, _ = obs.envelope_gradients(geo, static, state, cache, precision=gprec)
    return e, obs.forces_from_dR(dR)


def stress(system: System, state: SCFState | None = None, **scf_kwargs):
    """sigma = -(1/Omega) dF/deps, symmetrised, ABACUS sign (api.py:131-146)."""
    kw, gprec = _split_kwargs(dict(scf_kwargs))
    geo, static = system.geo, system.static
    cache = build_geometry_cache(geo, static)
    state = solve_scf(geo, static, cache=cache, **kw) if state is None else state
    _, deps = obs.envelope_gradients(geo, static, state, cache, precision=gprec)
    return obs.stress_from_deps(volume(geo.lattice), deps)


def energy_decomposition(system: System, state: SCFState | None = None, active=None):
    """Seven tagged terms (api.py:149-152)."""
    state = scf(system) if state is None else state
    kw = {} if active is None else {"active": active}
    return obs.energy_terms(system.geo, system.static, state, **kw)


def setup_from_case(case_dir):
    """System from an ABACUS case directory (INPUT / KPT / STRU + UPF), api.py:48-51."""
    from .abacus import setup_from_case as _from_case
    return _from_case(case_dir)
