"""SCF on the GPU: effective potential, eigensolvers, occupations, DIIS, driver.

Mirrors src/addft/solver/scf.py:81-92 (effective_potential), 171-183
(scf_map), 226-282 (residual, DIIS driver with 4 polish steps), mixer.py:23-82
(DIIS m = 8) and davidson.py:20-77 (block Davidson with the ABACUS
preconditioner and restarts).  Every H psi, density, Hartree, XC and
occupation step runs in libaddft_gb300 kernels; torch supplies the FP64
subspace linear algebra (cuBLAS GEMMs, cuSOLVER eigh / QR) on the device.

Precision modes:
  "fp64"  plain FP64 kernels everywhere (the oracle form);
  "fp32"  FP32 H psi inside Davidson with FP64 refinement: the Ritz pairs
          are re-anchored on an FP64 H X every SCF iteration once the
          density residual is small, and the correction vectors' H c stay
          FP32 (their error enters the Rayleigh quotient at second order).
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import ops
from .geometry import Cell
from .system import GeometryCache, SCFState, Static, build_geometry_cache


# ---------------------------------------------------------------------------
# effective potential  (scf.py:81-92)
# ---------------------------------------------------------------------------

def effective_potential(static: Static, cache: GeometryCache, rho: torch.Tensor, rho_dc=None):
    dev = static.device()
    v_h, e_h = ops.hartree(dev.wfc, cache.bvec, cache.omega, rho)
    v_xc, v_eff, sums = ops.xc_lda(rho, rho_dc=rho_dc, v_loc=cache.v_loc_r, v_h=v_h, want_vxc=True,
                                   want_veff=True)
    return v_eff, {"v_h": v_h, "v_xc": v_xc, "e_h": e_h, "xc_sums": sums}


def initial_density(static: Static, cache: GeometryCache) -> torch.Tensor:
    return torch.full((static.basis.nfft,), static.nelec / cache.omega, dtype=torch.float64, device="cuda")


def density_residual(static: Static, cache: GeometryCache, rho_new, rho_old) -> torch.Tensor:
    """sum |drho| Omega/N/N_e (scf.py:226-229), as a device scalar."""
    return torch.sum(torch.abs(rho_new - rho_old)) * (cache.omega / static.basis.nfft / static.nelec)


def wocc_of(static: Static, occ: torch.Tensor) -> torch.Tensor:
    return static.kweights_t()[:, None] * occ * static.spin_degeneracy


def density_of(static: Static, cache: GeometryCache, psi, occ) -> torch.Tensor:
    return ops.density(static.device().wfc, psi, wocc_of(static, occ), cache.omega)


# ---------------------------------------------------------------------------
# H psi in the requested precision
# ---------------------------------------------------------------------------

class HApply:
    """H psi for one k point on row-vector blocks (m, nG) complex128 in, complex128 out."""

    def __init__(self, static: Static, cache: GeometryCache, v_eff: torch.Tensor, precision: str = "fp64"):
        self.static, self.cache = static, cache
        self.plan = static.device().wfc
        self.v64 = v_eff
        self.v32 = v_eff.to(torch.float32) if precision == "fp32" else None
        self.precision = precision
        self.napply = 0

    def apply(self, k: int, Q: torch.Tensor, fp64: bool = None) -> torch.Tensor:
        use64 = (self.precision == "fp64") if fp64 is None else fp64
        c = self.cache
        self.napply += Q.shape[0]
        if use64:
            out = ops.hpsi(self.plan, Q.unsqueeze(0).contiguous(), c.kin[k:k + 1], self.v64,
                           c.proj[k:k + 1], c.dion)
            return out[0]
        proj32, dion32, kin32 = c.f32()
        out = ops.hpsi(self.plan, Q.to(torch.complex64).unsqueeze(0).contiguous(), kin32[k:k + 1], self.v32,
                       proj32[k:k + 1], dion32)
        return out[0].to(torch.complex128)


# ---------------------------------------------------------------------------
# eigensolvers
# ---------------------------------------------------------------------------

def _hermitize(T):
    return 0.5 * (T + T.conj().transpose(-1, -2))


def dense_lowest(H: HApply, k: int, nband: int):
    """Full-space Rayleigh-Ritz: H = H psi(I), FP64 cuSOLVER eigh (solver/eigh.py:30-41)."""
    nG = H.plan.nG
    eye = torch.eye(nG, dtype=torch.complex128, device="cuda")
    Hm = H.apply(k, eye, fp64=True).transpose(0, 1)       # column j = H e_j
    w, v = torch.linalg.eigh(_hermitize(Hm))
    return w[:nband], v[:, :nband].transpose(0, 1).contiguous(), 0.0


def _precond(lam, diag, kind="abacus", alpha=1.0):
    """ABACUS preconditioner 0.5(1 + x + sqrt(1 + (x-1)^2)), x = |h_diag - lambda| (davidson.py:20-29)."""
    if kind == "identity":
        return torch.ones((lam.shape[0], diag.shape[0]), dtype=torch.float64, device=diag.device)
    d = diag[None, :] - lam[:, None]
    if kind == "kinetic":
        return torch.where(torch.abs(d) > 1e-6, d, torch.ones_like(d))
    x = torch.abs(d)
    base = 0.5 * (1.0 + x + torch.sqrt(1.0 + (x - 1.0) ** 2))
    return torch.clamp(base, min=1e-6) ** alpha


def _orth_rows(R: torch.Tensor) -> torch.Tensor:
    q, _ = torch.linalg.qr(R.transpose(0, 1))
    return q.transpose(0, 1).contiguous()


def _project_out(R, Q):
    for _ in range(2):
        R = R - (R @ Q.conj().transpose(0, 1)) @ Q
    return R


@dataclass
class DavidsonResult:
    eig: torch.Tensor
    vec: torch.Tensor
    resid: float
    iters: int


def davidson_lowest(H: HApply, k: int, X0: torch.Tensor, nband: int, diag: torch.Tensor, max_sub: int,
                    max_iter: int, tol: float, precond: str = "abacus"):
    """Block Davidson for the lowest nband states of H at k (davidson.py:32-77), rows = vectors.

    Stops when the largest residual norm |H x - lambda x| drops below tol.  Only
    the residuals of unconverged bands expand the subspace; the subspace is
    orthonormalised twice against itself and restarted from the Ritz vectors
    when it would exceed max_sub.
    """
    nb = int(nband)
    nG = X0.shape[1]
    max_sub = min(int(max_sub), nG)
    Q = _orth_rows(X0)
    HQ = H.apply(k, Q)
    lam, resid, it = None, float("inf"), 0
    X = None
    for it in range(1, max_iter + 1):
        T = Q.conj() @ HQ.transpose(0, 1)
        w, U = torch.linalg.eigh(_hermitize(T))
        Qn = U.transpose(0, 1) @ Q
        HQn = U.transpose(0, 1) @ HQ
        X, HX, lam = Qn[:nb], HQn[:nb], w[:nb]
        R = HX - lam[:, None] * X
        rn = torch.linalg.vector_norm(R, dim=1)
        resid = float(rn.max())
        if resid < tol or it == max_iter:
            break
        active = rn > 0.1 * tol
        R = R[active] / _precond(lam[active], diag, precond)
        if Qn.shape[0] + R.shape[0] > max_sub:
            Qn, HQn = X, HX
        qadd = _orth_rows(_project_out(R, Qn))
        qadd = _orth_rows(_project_out(qadd, Qn))
        Q = torch.cat([Qn, qadd], 0)
        HQ = torch.cat([HQn, H.apply(k, qadd)], 0)
    return DavidsonResult(eig=lam, vec=X.contiguous(), resid=resid, iters=it)


def refine_lowest(H: HApply, k: int, X: torch.Tensor, nband: int, diag: torch.Tensor, iters: int, tol: float,
                  precond: str = "abacus", inner: int = 3):
    """FP64-anchored refinement of Ritz pairs (defect correction).

    Each outer pass computes H X in FP64, the exact residual R = H X - lambda X
    and then runs ``inner`` Davidson expansions whose correction blocks C are
    applied in the working precision.  In the projected matrix only the C-C
    blocks carry the FP32 error: the X-C blocks come from the FP64 H X (H is
    Hermitian), so the Ritz values are exact to first order in the correction.
    """
    nb = int(nband)
    lam, resid, it = None, float("inf"), 0
    X = _orth_rows(X)
    for it in range(1, iters + 1):
        HX = H.apply(k, X, fp64=True)
        T = X.conj() @ HX.transpose(0, 1)
        w, U = torch.linalg.eigh(_hermitize(T))
        X = U.transpose(0, 1) @ X
        HX = U.transpose(0, 1) @ HX
        lam = w[:nb]
        R = HX - lam[:, None] * X
        rn = torch.linalg.vector_norm(R, dim=1)
        resid = float(rn.max())
        if resid < tol or it == iters:
            break
        Q, HQ = X, HX
        Xi, HXi, lami, Ri = X, HX, lam, R
        for _ in range(inner):
            C = _orth_rows(_project_out(Ri / _precond(lami, diag, precond), Q))
            C = _orth_rows(_project_out(C, Q))
            HC = H.apply(k, C)
            Q = torch.cat([Q, C], 0)
            HQ = torch.cat([HQ, HC], 0)
            T = Q.conj() @ HQ.transpose(0, 1)
            # rows/cols of the anchor block from the FP64 H X: <c|H|x> = conj(<x|H c>)
            T[nb:, :nb] = Q[nb:].conj() @ HX.transpose(0, 1)
            T[:nb, nb:] = T[nb:, :nb].conj().transpose(0, 1)
            w, U = torch.linalg.eigh(_hermitize(T))
            Ub = U[:, :nb].transpose(0, 1)
            Xi, HXi, lami = Ub @ Q, Ub @ HQ, w[:nb]
            Ri = HXi - lami[:, None] * Xi
        X = Xi.contiguous()
    return DavidsonResult(eig=lam, vec=X.contiguous(), resid=resid, iters=it)


# ---------------------------------------------------------------------------
# DIIS mixer (mixer.py:23-82), on device tensors
# ---------------------------------------------------------------------------

class DIISMixer:
    def __init__(self, m: int = 8, beta: float = 0.5):
        self.m, self.beta = int(m), float(beta)
        self.rins, self.routs = [], []

    def reset(self):
        self.rins.clear()
        self.routs.clear()

    def __call__(self, rho_in, rho_out):
        self.rins.append(rho_in)
        self.routs.append(rho_out)
        if len(self.rins) > self.m:
            self.rins.pop(0)
            self.routs.pop(0)
        if len(self.rins) == 1:
            return rho_in + self.beta * (rho_out - rho_in)
        n = len(self.rins)
        rins = torch.stack(self.rins)
        res = torch.stack(self.routs) - rins
        B = torch.zeros((n + 1, n + 1), dtype=torch.float64, device=rins.device)
        B[:n, :n] = res @ res.T
        B[:n, n] = -1.0
        B[n, :n] = -1.0
        B = B + torch.eye(n + 1, dtype=torch.float64, device=rins.device) * 1e-12
        rhs = torch.zeros(n + 1, dtype=torch.float64, device=rins.device)
        rhs[n] = -1.0
        c = torch.nan_to_num(torch.linalg.solve(B, rhs)[:n], nan=0.0, posinf=0.0, neginf=0.0)
        new = c @ (rins + self.beta * res)
        if not bool(torch.isfinite(new).all()):
            self.reset()
            return rho_in + self.beta * (rho_out - rho_in)
        return new


# ---------------------------------------------------------------------------
# SCF
# ---------------------------------------------------------------------------

@dataclass
class EigenOptions:
    solver: str = "auto"          # auto | dense | davidson
    precision: str = "fp64"       # fp64 | fp32
    dense_max_nG: int = 1500
    max_sub: int = 0              # 0 -> max(48, 4 nband) (scf.py:318-320)
    max_iter: int = 60
    refine_iters: int = 4
    precond: str = "abacus"


class Eigensolver:
    """Lowest nband Ritz pairs of H[v] per k with warm starts across SCF steps."""

    def __init__(self, static: Static, cache: GeometryCache, opts: EigenOptions):
        self.static, self.cache, self.opts = static, cache, opts
        nG = static.basis.nG
        self.dense = opts.solver == "dense" or (opts.solver == "auto" and nG <= opts.dense_max_nG)
        self.X = None
        self.napply64 = 0
        self.napply32 = 0

    def _start(self, nG, nb):
        # cold start: the lowest-|G| plane waves (scf.py:359-360)
        X = torch.zeros((self.static.nk, nb, nG), dtype=torch.complex128, device="cuda")
        idx = torch.arange(nb, device="cuda")
        X[:, idx, idx] = 1.0
        return X

    def solve(self, v_eff: torch.Tensor, tol: float, refine: bool = False):
        st, c, o = self.static, self.cache, self.opts
        nb, nk, nG = st.nband, st.nk, st.basis.nG
        H = HApply(st, c, v_eff, "fp64" if self.dense else o.precision)
        eig = torch.empty((nk, nb), dtype=torch.float64, device="cuda")
        vec = torch.empty((nk, nb, nG), dtype=torch.complex128, device="cuda")
        resid = 0.0
        if self.X is None:
            self.X = self._start(nG, nb)
        for k in range(nk):
            if self.dense:
                w, v, r = dense_lowest(H, k, nb)
                self.napply64 += nG
            else:
                max_sub = o.max_sub or max(48, 4 * nb)
                diag = c.kin[k] + torch.mean(v_eff)
                if refine and o.precision == "fp32":
                    res = refine_lowest(H, k, self.X[k], nb, diag, o.refine_iters, tol, o.precond)
                    self.napply64 += nb * res.iters
                    H.napply -= nb * res.iters
                else:
                    res = davidson_lowest(H, k, self.X[k], nb, diag, max_sub, o.max_iter, tol, o.precond)
                w, v, r = res.eig, res.vec, res.resid
            eig[k], vec[k] = w, v
            resid = max(resid, r)
        if not self.dense:
            if o.precision == "fp32":
                self.napply32 += H.napply
            else:
                self.napply64 += H.napply
        self.X = vec.clone()
        return eig, vec, resid


def occupations(static: Static, eig):
    return ops.occupations(eig, static.kweights_t(), static.nelec, static.sigma, static.spin_degeneracy)


def scf_step(static, cache, rho, eigs: Eigensolver, tol_eig):
    v_eff, _ = effective_potential(static, cache, rho)
    eig, psi, eres = eigs.solve(v_eff, tol_eig)
    occ, mu = occupations(static, eig)
    rho_out = density_of(static, cache, psi, occ)
    return rho_out, eig, psi, occ, mu, eres


def scf_map(geo: Cell, static: Static, rho_r, cache=None, precision="fp64"):
    """n -> H[n] -> lowest states -> occupations -> n' (scf.py:171-183)."""
    cache = cache or build_geometry_cache(geo, static)
    eigs = Eigensolver(static, cache, EigenOptions(precision=precision))
    return scf_step(static, cache, rho_r, eigs, 1e-11)[0]


def solve_scf(geo: Cell, static: Static, alpha=0.9, gg0=0.5, tol=1e-10, max_iter=200, verbose=False,
              mixer="diis", beta=0.5, driver="auto", eigh_solver="auto", precision="fp64",
              cache: GeometryCache = None, rho0=None, polish: int = 4, stats: dict = None) -> SCFState:
    """DIIS SCF with 4 unmixed polish steps and a final diagonalisation (scf.py:239-282).

    ``eigh_solver`` in {"auto", "dense", "davidson"}; ``precision`` in {"fp64", "fp32"}.
    ``alpha``, ``gg0``, ``driver`` are accepted for signature parity with the reference.
    """
    del alpha, gg0, driver
    if mixer != "diis":
        raise ValueError("only the DIIS mixer is provided")
    cache = cache or build_geometry_cache(geo, static)
    opts = EigenOptions(solver=eigh_solver, precision=precision)
    eigs = Eigensolver(static, cache, opts)
    rho = initial_density(static, cache) if rho0 is None else rho0
    mix = DIISMixer(m=8, beta=beta)
    prev, res, it = 1e9, 1.0, 0
    fp32 = precision == "fp32" and not eigs.dense
    for it in range(1, max_iter + 1):
        tol_eig = max(min(1e-3, 0.1 * res), 1e-11)
        refine = fp32 and res < 1e-4
        v_eff, _ = effective_potential(static, cache, rho)
        eig, psi, eres = eigs.solve(v_eff, tol_eig, refine=refine)
        occ, mu = occupations(static, eig)
        rho_out = density_of(static, cache, psi, occ)
        res = float(density_residual(static, cache, rho_out, rho))
        if res > prev * 1.5:
            mix.reset()
        prev = res
        rho = mix(rho, rho_out)
        if verbose:
            print(f"  scf {it:3d}  drho={res:.3e}  eigres={eres:.2e}")
        if res < tol:
            break
    for _ in range(polish):
        v_eff, _ = effective_potential(static, cache, rho)
        eig, psi, eres = eigs.solve(v_eff, 1e-11, refine=fp32)
        occ, mu = occupations(static, eig)
        rho_new = density_of(static, cache, psi, occ)
        res = float(density_residual(static, cache, rho_new, rho))
        rho = rho_new
        if res < 1e-14:
            break
    v_eff, _ = effective_potential(static, cache, rho)
    eig, psi, eres = eigs.solve(v_eff, 1e-11, refine=fp32)
    occ, mu = occupations(static, eig)
    if stats is not None:
        stats.update(napply64=eigs.napply64, napply32=eigs.napply32, iters=it, eig_resid=eres)
    return SCFState(psi=psi, eig=eig, occ=occ, mu=mu, rho_r=rho, n_iter=it, residual=res)
