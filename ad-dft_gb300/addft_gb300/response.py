"""Matrix-free linear response of the SCF map and the fixed-point adjoint.

Mirrors src/addft/physics/response.py:42-121 (make_response),
diff/implicit.py:32-110 (implicit_grad, forces_from_grad, stress_from_grad)
and observables/constraint.py:26-44 (delta_q, delta_q_grad).

The reference differentiates the map F(n) = n_out[H[n]] with a dense
eigen-decomposition of the full H (all nG states).  Here the response to a
local potential change dv is built without it:

  * for band pairs inside an extended window -- the nband states plus empty
    buffer states above them, computed at the converged potential (the whole
    remaining spectrum when the basis is small enough for a dense
    eigensolve) -- the first-order coefficients M_mn / (e_n - e_m) (pairs
    with |e_n - e_m| <= tol dropped, as the reference does) come from
    M = C^H (dv C), dv C by the FP64 H psi kernels.  The buffer carries the
    states that are nearly degenerate with the top of the band window;
  * the rest of the spectrum enters through Sternheimer equations
    (H - e_n) x_n = -Q dv c_n on range(Q), Q = 1 - C C^H - C_b C_b^H, solved
    by preconditioned conjugate gradients with FP64 H psi (H - e_n is
    positive on range(Q) because the extended window holds the lowest states);
  * occupations follow f = 1 / (1 + exp((e - mu)/sigma)):
    df_n = -f_n (1 - f_n)/sigma (de_n - dmu), with dmu fixing the electron
    count over all k points.  The reference writes +f(1-f)/sigma with a
    per-k dmu (response.py:104-107); its fixtures have f(1-f) ~ 0, and the
    sign used here is the derivative of its own occupation function
    (physics/occupation.py:18-20), checked against central differences.

The Hartree + XC kernel K and the independent-particle response chi0 are
both symmetric, so the transposed Jacobian of the map is K chi0 and the
adjoint (I - K chi0) lambda = dL/dn needs no transposition machinery.  The
explicit geometry derivative lambda^T dF/dtheta at fixed n is
Tr[dH/dtheta dP_lambda] (dP_lambda = density-matrix response to the
potential lambda) plus the 1/Omega normalisation of n_out; its local,
nonlocal and kinetic parts run through the envelope-gradient kernels with
cross terms obtained by polarisation, <a|O|b> + <b|O|a> =
<a+b|O|a+b> - <a|O|a> - <b|O|b>.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import ops
from .geometry import Cell
from .solver import HApply, _precond, davidson_lowest, dense_lowest, effective_potential, wocc_of
from .system import GeometryCache, SCFState, Static, build_geometry_cache

FOUR_PI = 4.0 * np.pi


@dataclass
class Perturbation:
    dpsi: torch.Tensor      # (nk, nb, nG) complex128, first-order band change
    df: torch.Tensor        # (nk, nb) occupation change
    drho: torch.Tensor      # (N,) density change


class Response:
    """Linear response of the SCF map at a converged state (FP64)."""

    def __init__(self, geo: Cell, static: Static, state: SCFState, cache: GeometryCache = None,
                 tol: float = 1e-6, cg_tol: float = 1e-13, cg_maxiter: int = 400, nbuf: int = None,
                 dense_max_nG: int = 1500):
        self.geo, self.static, self.state = geo, static, state
        self.cache = cache or build_geometry_cache(geo, static)
        self.tol, self.cg_tol, self.cg_maxiter = float(tol), float(cg_tol), int(cg_maxiter)
        self.dev = static.device()
        self.v_eff, _ = effective_potential(static, self.cache, state.rho_r)
        self.H = HApply(static, self.cache, self.v_eff, "fp64")
        self.C = state.psi.to(torch.complex128)
        self.eig = state.eig.to(torch.float64)
        self.f = state.occ.to(torch.float64)
        self.kw = static.kweights_t()
        sigma = static.sigma
        self.fprime = self.f * (1.0 - self.f) / sigma if sigma > 1e-6 else torch.zeros_like(self.f)
        self.kin0 = torch.zeros((1, self.C.shape[2]), dtype=torch.float64, device="cuda")
        self.cg_iters = 0
        self._buffer(nbuf, dense_max_nG)

    def _buffer(self, nbuf, dense_max_nG):
        """Empty states above the window: all of them (dense) or nbuf by FP64 Davidson,
        orthogonalised against the SCF bands."""
        nk, nb, nG = self.C.shape
        self.full = nG <= dense_max_nG
        self.Cb, self.eb = [], []
        for k in range(nk):
            if self.full:
                w, v, _ = dense_lowest(self.H, k, nG)
                w, v = w[nb:], v[nb:]
            else:
                m = nbuf or max(8, nb // 4)
                diag = self.cache.kin[k] + torch.mean(self.v_eff)
                X0 = torch.cat([self.C[k], torch.randn((m + 4, nG), dtype=torch.complex128, device="cuda",
                                                       generator=torch.Generator("cuda").manual_seed(k))], 0)
                wts = torch.ones(nb + m + 4, dtype=torch.float64, device="cuda")
                wts[nb + m:] = 0.0
                r = davidson_lowest(self.H, k, X0, nb + m + 4, diag, 3 * (nb + m + 4), 300, 1e-10, weights=wts)
                w, v = r.eig[nb:nb + m], r.vec[nb:nb + m]
            v = self._project(k, v)
            v = self._project(k, v)
            S = v.conj() @ v.transpose(0, 1)
            L = torch.linalg.cholesky(0.5 * (S + S.conj().transpose(0, 1)))
            v = torch.linalg.solve_triangular(L, v, upper=False)
            self.Cb.append(v.contiguous())
            self.eb.append(w.to(torch.float64))

    # -- operators -----------------------------------------------------------
    def kernel(self, dn: torch.Tensor) -> torch.Tensor:
        """K dn = v_H[dn] + f_xc(n) dn on the wavefunction shell (response.py:70-76)."""
        c = self.cache
        v_h, _ = ops.hartree(self.dev.wfc, c.bvec, c.omega, dn)
        return v_h + ops.xc_lda_vjp(self.state.rho_r, dn)

    def _local(self, k: int, X: torch.Tensor, dv: torch.Tensor) -> torch.Tensor:
        return ops.hpsi(self.dev.wfc, X.unsqueeze(0).contiguous(), self.kin0, dv)[0]

    def _project(self, k: int, V: torch.Tensor, buffer: bool = False) -> torch.Tensor:
        C = self.C[k]
        V = V - (V @ C.conj().transpose(0, 1)) @ C
        if buffer and self.Cb[k].shape[0]:
            B = self.Cb[k]
            V = V - (V @ B.conj().transpose(0, 1)) @ B
        return V

    def _sternheimer(self, k: int, b: torch.Tensor, eps: torch.Tensor) -> torch.Tensor:
        """Rows x_n in range(Q) with Q (H - eps_n) x_n = b_n, by preconditioned CG."""
        if b.shape[0] == 0:
            return b
        diag = self.cache.kin[k] + torch.mean(self.v_eff)
        Pinv = 1.0 / _precond(eps, diag)
        x = torch.zeros_like(b)
        r = b.clone()
        bn = torch.linalg.vector_norm(b, dim=1)
        z = self._project(k, r * Pinv, True)
        p = z.clone()
        rz = torch.sum(torch.conj(r) * z, dim=1).real
        for it in range(self.cg_maxiter):
            Ap = self._project(k, self.H.apply(k, p, fp64=True) - eps[:, None] * p, True)
            pAp = torch.sum(torch.conj(p) * Ap, dim=1).real
            alpha = torch.where(pAp > 0, rz / torch.where(pAp > 0, pAp, 1.0), torch.zeros_like(rz))
            x = x + alpha[:, None] * p
            r = r - alpha[:, None] * Ap
            self.cg_iters += 1
            if bool(torch.all(torch.linalg.vector_norm(r, dim=1) <= self.cg_tol * torch.clamp(bn, min=1e-300))):
                break
            z = self._project(k, r * Pinv, True)
            rz_new = torch.sum(torch.conj(r) * z, dim=1).real
            beta = torch.where(rz > 0, rz_new / torch.where(rz > 0, rz, 1.0), torch.zeros_like(rz))
            p = z + beta[:, None] * p
            rz = rz_new
        return x

    def perturb(self, dv: torch.Tensor) -> Perturbation:
        """First-order band, occupation and density change for a local potential change dv(r)."""
        st, c = self.static, self.cache
        nk, nb, nG = self.C.shape
        dpsi = torch.zeros_like(self.C)
        de = torch.zeros((nk, nb), dtype=torch.float64, device="cuda")
        for k in range(nk):
            C, eps = self.C[k], self.eig[k]
            VC = self._local(k, C, dv)
            M = C.conj() @ VC.transpose(0, 1)                   # M[m, n] = <c_m|dv|c_n>
            M = 0.5 * (M + M.conj().transpose(0, 1))
            de[k] = torch.diagonal(M).real
            d = eps[None, :] - eps[:, None]                      # d[m, n] = e_n - e_m
            off = torch.abs(d) > self.tol
            coef = torch.where(off, M / torch.where(off, d, torch.ones_like(d)), torch.zeros_like(M))
            dpsi[k] = coef.transpose(0, 1) @ C                   # in-window part, row n
            B, eb = self.Cb[k], self.eb[k]
            if B.shape[0]:
                Mb = B.conj() @ VC.transpose(0, 1)                # <b_m|dv|c_n>
                db = eps[None, :] - eb[:, None]
                offb = torch.abs(db) > self.tol
                cb = torch.where(offb, Mb / torch.where(offb, db, torch.ones_like(db)), torch.zeros_like(Mb))
                dpsi[k] += cb.transpose(0, 1) @ B
            if not self.full:
                act = self.f[k] * self.kw[k] > 1e-14 * float(torch.max(self.f[k]))
                idx = torch.nonzero(act).flatten()
                if idx.numel():
                    b = -self._project(k, VC[idx], True)
                    dpsi[k, idx] += self._sternheimer(k, b, eps[idx])
        if st.sigma > 1e-6:
            wf = self.kw[:, None] * self.fprime
            dmu = torch.sum(wf * de) / (torch.sum(wf) + 1e-300)
            df = -self.fprime * (de - dmu)
        else:
            df = torch.zeros_like(de)
        drho = self._cross_density(dpsi) + ops.density(self.dev.wfc, self.C, wocc_of(st, df), c.omega)
        return Perturbation(dpsi=dpsi, df=df, drho=drho)

    def _cross_density(self, dpsi: torch.Tensor) -> torch.Tensor:
        """sum_n w f_n 2 Re(conj(psi_n(r)) dpsi_n(r)) / Omega by polarisation."""
        st, c = self.static, self.cache
        w = wocc_of(st, self.f)
        s = 1.0 / max(float(torch.max(torch.abs(dpsi))), 1e-300) * float(torch.max(torch.abs(self.C)))
        b = s * dpsi
        dens = lambda x: ops.density(self.dev.wfc, x, w, c.omega)  # noqa: E731
        return (dens(self.C + b) - dens(self.C) - dens(b)) / s

    def chi0(self, dv: torch.Tensor) -> torch.Tensor:
        return self.perturb(dv).drho

    def apply(self, dn: torch.Tensor) -> torch.Tensor:
        """(dF/dn) dn = chi0 K dn, the reference's make_response apply."""
        return self.chi0(self.kernel(dn))

    def apply_t(self, y: torch.Tensor) -> torch.Tensor:
        """(dF/dn)^T y = K chi0 y (K and chi0 are symmetric)."""
        return self.kernel(self.chi0(y))


def make_response(geo: Cell, static: Static, state: SCFState, tol: float = 1e-6, cache=None):
    """Pure function dn -> (dF/dn) dn (response.py:42-121)."""
    return Response(geo, static, state, cache=cache, tol=tol).apply


# ---------------------------------------------------------------------------
# adjoint
# ---------------------------------------------------------------------------

def bicgstab(op, b: torch.Tensor, rtol: float = 1e-10, maxiter: int = 200):
    """BiCGSTAB for op(x) = b on device vectors (implicit.py:53-65)."""
    x = torch.zeros_like(b)
    r = b - op(x)
    rhat = r.clone()
    rho = alpha = omega = 1.0
    v = torch.zeros_like(b)
    p = torch.zeros_like(b)
    bn = float(torch.linalg.vector_norm(b))
    it = 0
    if bn == 0.0:
        return x, it   # b = 0: x = 0 exactly
    for it in range(1, maxiter + 1):
        rho_new = float(torch.dot(rhat, r))
        if rho_new == 0.0:
            break      # breakdown (r orthogonal to the shadow residual): the caller checks the residual
        beta = (rho_new / rho) * (alpha / omega) if it > 1 else 0.0
        p = r + beta * (p - omega * v) if it > 1 else r.clone()
        v = op(p)
        rv = float(torch.dot(rhat, v))
        if rv == 0.0:
            break
        alpha = rho_new / rv
        s = r - alpha * v
        if float(torch.linalg.vector_norm(s)) <= rtol * bn:
            x = x + alpha * p
            r = s
            break
        t = op(s)
        omega = float(torch.dot(t, s)) / max(float(torch.dot(t, t)), 1e-300)
        x = x + alpha * p + omega * s
        r = s - omega * t
        rho = rho_new
        if float(torch.linalg.vector_norm(r)) <= rtol * bn or omega == 0.0:
            break      # converged, or omega = 0 (the next beta would divide by it)
    return x, it


def _hartree_strain_cross(static: Static, cache: GeometryCache, n1: torch.Tensor, n2: torch.Tensor):
    """d/deps of Omega sum_G 4 pi Re(n1(G) conj(n2(G))) / G^2 on the wavefunction
    shell with n1(G) and Omega n2(G) fixed: sum 4 pi Re(n1 conj(Omega n2)) 2 G_a G_b / G^4."""
    plan = static.device().wfc
    om = cache.omega
    g1 = ops.real_to_psi(plan, n1.to(torch.complex128), om) / np.sqrt(om)
    g2 = ops.real_to_psi(plan, n2.to(torch.complex128), om) / np.sqrt(om)
    G = torch.as_tensor(static.basis.miller.astype(np.float64) @ cache.bvec, device="cuda")
    q2 = torch.sum(G * G, dim=1)
    ok = q2 > 1e-14
    w = torch.where(ok, FOUR_PI * torch.real(g1 * torch.conj(g2)) * om * 2.0 / torch.where(ok, q2 * q2, 1.0),
                    torch.zeros_like(q2))
    return (G * w[:, None]).transpose(0, 1) @ G


def _map_theta_vjp(resp: Response, lam: torch.Tensor):
    """lambda^T dF/dtheta at fixed n: (dR (nat, 3), deps (3, 3)) on the device."""
    st, c, state = resp.static, resp.cache, resp.state
    dev = resp.dev
    nat = st.natom
    # lambda^T n = sum_r lambda(r) n(r) while <a|v|b> = (Omega/N) sum_r v conj(a) b: the
    # potential reciprocal to the covector lambda is (N/Omega) lambda
    pt = resp.perturb(lam * (st.basis.nfft / c.omega))
    # local potential (V_loc) part: int dV_loc/dtheta drho_lambda (frozen coefficients)
    dg = ops.density_gradients(dev.wfc, dev.rho, c.bvec, c.omega, c.pos, st.psp, pt.drho)
    dR = dg[5:5 + 3 * nat].reshape(nat, 3).clone()
    deps = dg[5 + 3 * nat + 9:].reshape(3, 3).clone()
    # Hartree potential of the fixed input density
    deps = deps + _hartree_strain_cross(st, c, state.rho_r, pt.drho)
    # nonlocal and kinetic: band cross terms by polarisation, occupation terms directly
    w = wocc_of(st, resp.f)
    wdf = wocc_of(st, pt.df)
    s = float(torch.max(torch.abs(resp.C))) / max(float(torch.max(torch.abs(pt.dpsi))), 1e-300)
    b = s * pt.dpsi

    def nl(psi, wocc):
        out = ops.nonlocal_gradients(dev.wfc, c.bvec, c.omega, st.kpts, c.pos, st.psp, psi, wocc, c.dion)
        return out[1:1 + 3 * nat].reshape(nat, 3), out[1 + 3 * nat:].reshape(3, 3)

    def kin(psi, wocc):
        return ops.kinetic_stress(dev.wfc, c.bvec, st.kpts, psi, wocc).reshape(3, 3)

    a1, e1 = nl(resp.C + b, w)
    a2, e2 = nl(resp.C, w)
    a3, e3 = nl(b, w)
    a4, e4 = nl(resp.C, wdf)
    dR = dR + (a1 - a2 - a3) / s + a4
    deps = deps + (e1 - e2 - e3) / s + e4
    deps = deps + (kin(resp.C + b, w) - kin(resp.C, w) - kin(b, w)) / s + kin(resp.C, wdf)
    # n_out carries 1/Omega: d ln Omega / d eps_ab = delta_ab
    rho_out = ops.density(dev.wfc, resp.C, w, c.omega)
    deps = deps - float(torch.dot(lam, rho_out)) * torch.eye(3, dtype=torch.float64, device="cuda")
    return dR, deps


DENSE_MAX_NFFT = 4096


def _solve_adjoint(resp: Response, g_n: torch.Tensor, mode: str, rtol: float):
    """(I - dF/dn)^T lambda = g_n.  ``matrix_free``: BiCGSTAB on the transposed apply
    (implicit.py:53-65); ``dense``: the transposed Jacobian assembled column by column
    from the same apply and solved directly (implicit.py:45-50, a diagnostic for small
    boxes; build_jacobian at response.py:124-128)."""
    op = lambda y: y - resp.apply_t(y)  # noqa: E731
    if mode == "dense":
        n = int(g_n.numel())
        if n > DENSE_MAX_NFFT:
            raise ValueError(f"adjoint_mode='dense' assembles an {n} x {n} Jacobian; "
                             f"it is limited to boxes of <= {DENSE_MAX_NFFT} points")
        eye = torch.eye(n, dtype=torch.float64, device=g_n.device)
        at = torch.stack([op(eye[j]) for j in range(n)], dim=1)     # column j = A^T e_j
        lam = torch.linalg.solve(at, g_n)
        nit = n
    elif mode == "matrix_free":
        lam, nit = bicgstab(op, g_n, rtol=rtol)
    else:
        raise ValueError(f"unknown adjoint mode {mode!r} (matrix_free or dense)")
    res = float(torch.linalg.vector_norm(op(lam) - g_n) / (torch.linalg.vector_norm(g_n) + 1e-300))
    if res > 1e-6:
        raise RuntimeError(f"adjoint solve ({mode}) did not converge: residual {res:.3e}")
    return lam, nit, res


def implicit_grad(geo: Cell, static: Static, state: SCFState, g_n: torch.Tensor, dL_dR=None, dL_deps=None,
                  rtol: float = 1e-10, cache=None, return_diagnostics: bool = False, mode: str = "matrix_free"):
    """dL/dgeo for a scalar L(geo, n*) given dL/dn (g_n, device (N,)) and its explicit
    geometry derivatives at fixed n (implicit.py:32-87):

        (I - dF/dn)^T lambda = dL/dn,   dL/dtheta = dL/dtheta|_n* + lambda^T dF/dtheta.

    ``mode`` is the reference's adjoint_mode: "matrix_free" (BiCGSTAB) or "dense".
    Returns Cell(lattice = dL/dL at fixed frac, frac = dL/dfrac) as NumPy arrays.
    """
    resp = Response(geo, static, state, cache=cache)
    lam, nit, res = _solve_adjoint(resp, g_n, mode, rtol)
    dR, deps = _map_theta_vjp(resp, lam)
    dR = dR.cpu().numpy()
    deps = deps.cpu().numpy()
    if dL_dR is not None:
        dR = dR + np.asarray(dL_dR)
    if dL_deps is not None:
        deps = deps + np.asarray(dL_deps)
    lat = np.asarray(geo.lattice, dtype=np.float64)
    grad = Cell(lattice=np.linalg.inv(lat).T @ deps, frac=dR @ lat.T)
    if not return_diagnostics:
        return grad
    return grad, {"adjoint_residual": res, "bicgstab_iters": nit, "sternheimer_cg_iters": resp.cg_iters,
                  "lam_norm": float(torch.linalg.vector_norm(lam)), "g_norm": float(torch.linalg.vector_norm(g_n)),
                  "dR": dR, "deps": deps}


def forces_from_grad(geo: Cell, grad_cell) -> np.ndarray:
    """F = -dE/dR with dE/dR = dE/dfrac inv(L)^T (implicit.py:96-103)."""
    return -(np.asarray(grad_cell.frac) @ np.linalg.inv(np.asarray(geo.lattice)).T)


def stress_from_grad(omega: float, grad_eps) -> np.ndarray:
    """sigma = -(1/Omega) dE/deps (implicit.py:106-113)."""
    return -np.asarray(grad_eps) / omega


def energy_implicit_grad(geo: Cell, static: Static, state: SCFState, cache=None, mode: str = "matrix_free",
                         rtol: float = 1e-10, return_diagnostics: bool = False):
    """Gradient of the Mermin free energy by the fixed-point adjoint: the backward of the
    reference's ``make_energy(static, mode="adjoint")`` (api.py:114-116), which hands
    L(geo, state) = F(geo, state) to implicit_grad (implicit.py:32-87) with psi and the
    occupations held fixed and only n* following the fixed point.

    F(geo; psi, f, n) = sum f <psi|T + V_loc + V_NL + V_H[n] + V_xc[n]|psi> - E_H[n] + E_xc[n]
    - <psi|V_xc[n]|psi> + E_II - sigma g_s S  (energy.py:134-169); the two V_xc matrix
    elements are the same function of n and cancel.  With rho_psi the band density at
    fixed coefficients (rho_psi ~ 1/Omega under strain) and n the fixed density array:

      dL/dn_j = (Omega/N) (V_H[rho_psi] - V_H[n] + v_xc[n])_j,
      dR: V_loc (through rho_psi), V_NL and Ewald -- the envelope terms;
      deps: kinetic, V_loc, V_NL, Ewald as in the envelope, plus
            d/deps Omega sum_G 4 pi Re(n(G) conj(rho_psi(G)))/G^2  (n(G), Omega rho_psi(G) fixed)
            - E_H[n] delta - (1/2) Omega sum_G 4 pi |n(G)|^2 2 G_a G_b / G^4  + E_xc[n] delta,

    then lambda^T dF_map/dtheta is added by implicit_grad.  At the fixed point
    dL/dn = (Omega/N) v_xc[n] is not zero, so this is not the envelope gradient: it is the
    reference's adjoint-mode quantity (its docstring keeps energies on the envelope path).
    Returns Cell(lattice, frac) like implicit_grad (with diagnostics on request)."""
    from .observables import _ewald
    from .solver import density_of
    cache = cache or build_geometry_cache(geo, static)
    dev = static.device()
    nat = static.natom
    om = cache.omega
    scale = om / static.basis.nfft
    n = state.rho_r
    rho_psi = density_of(static, cache, state.psi, state.occ)
    vh_psi, _ = ops.hartree(dev.wfc, cache.bvec, om, rho_psi)
    vh_n, eh_n = ops.hartree(dev.wfc, cache.bvec, om, n)
    vxc_n, _, sums = ops.xc_lda(n)
    g_n = scale * (vh_psi - vh_n + vxc_n)
    wocc = wocc_of(static, state.occ)
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    deps = ops.kinetic_stress(dev.wfc, cache.bvec, static.kpts, state.psi, wocc).reshape(3, 3)
    dg = ops.density_gradients(dev.wfc, dev.rho, cache.bvec, om, cache.pos, static.psp, rho_psi)
    dR = dg[5:5 + 3 * nat].reshape(nat, 3).clone()
    deps = deps + dg[5 + 3 * nat + 9:].reshape(3, 3)
    deps = deps + _hartree_strain_cross(static, cache, n, rho_psi)
    deps = deps - eh_n[0] * eye - 0.5 * _hartree_strain_cross(static, cache, n, n)
    deps = deps + scale * (sums[0] + sums[1]) * eye
    nl = ops.nonlocal_gradients(dev.wfc, cache.bvec, om, static.kpts, cache.pos, static.psp, state.psi, wocc,
                                cache.dion)
    dR = dR + nl[1:1 + 3 * nat].reshape(nat, 3)
    deps = deps + nl[1 + 3 * nat:].reshape(3, 3)
    ew = _ewald(static, geo, cache)
    dR = dR + ew[1:1 + 3 * nat].reshape(nat, 3)
    deps = deps + ew[1 + 3 * nat:].reshape(3, 3)
    return implicit_grad(geo, static, state, g_n, dL_dR=dR.cpu().numpy(), dL_deps=deps.cpu().numpy(), rtol=rtol,
                         cache=cache, return_diagnostics=return_diagnostics, mode=mode)
