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

import os
from dataclasses import dataclass

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


def density_of(static: Static, cache: GeometryCache, psi, occ, fp32: bool = False) -> torch.Tensor:
    """n(r) = sum_k w_k sum_n f_n |psi_n(r)|^2 / Omega; ``fp32`` runs the FFTs of the
    band sum in FP32 (relative error ~1e-7, FP64 accumulation)."""
    if fp32:
        psi = psi.to(torch.complex64)
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
        self.kin0 = None

    def _apply64(self, k: int, Q: torch.Tensor) -> torch.Tensor:
        """FP64-accurate H Q.  The plain FP64 kernel form (precision "fp64") runs every term in
        FP64.  The FP32 arm's anchors take the local part from the FP64 kernels and the two
        projector contractions (becp = conj(beta) Q^T, H Q += (D becp)^T beta) from the
        double-float GEMM (~1e-14 relative, 3-4x the FP64 rate), like its subspace products."""
        c = self.cache
        Q = Q.contiguous()
        if self.precision != "fp32" or not DF_GEMM or c.proj.shape[1] == 0:
            return ops.hpsi(self.plan, Q.unsqueeze(0), c.kin[k:k + 1], self.v64, c.proj[k:k + 1], c.dion)[0]
        out = ops.hpsi(self.plan, Q.unsqueeze(0), c.kin[k:k + 1], self.v64)[0]
        beta = c.proj[k]                                            # (P, nG)
        becp = ops.zgemm_df(beta, Q.transpose(0, 1), conj_a=True)   # (P, m)
        db = c.dion.to(torch.complex128) @ becp                     # (P, m), P x P x m
        return out + ops.zgemm_df(db.transpose(0, 1), beta)         # (m, nG)

    def apply_native(self, k: int, Q: torch.Tensor) -> torch.Tensor:
        """H Q in the precision of Q (complex64 -> FP32 kernels, complex128 -> FP64-accurate)."""
        c = self.cache
        self.napply += Q.shape[0]
        if Q.dtype == torch.complex128:
            return self._apply64(k, Q)
        proj32, dion32, kin32 = c.f32()
        if self.v32 is None:
            self.v32 = self.v64.to(torch.float32)
        return ops.hpsi(self.plan, Q.unsqueeze(0).contiguous(), kin32[k:k + 1], self.v32, proj32[k:k + 1],
                        dion32)[0]

    def apply_local(self, k: int, Q: torch.Tensor, dv: torch.Tensor) -> torch.Tensor:
        """dv(r) Q with the FP32 kernels (no kinetic or nonlocal term); Q complex64."""
        self.napply += Q.shape[0]
        if self.kin0 is None:
            self.kin0 = torch.zeros((1, self.plan.nG), dtype=torch.float32, device=Q.device)
        return ops.hpsi(self.plan, Q.unsqueeze(0).contiguous(), self.kin0, dv)[0]

    def apply(self, k: int, Q: torch.Tensor, fp64: bool = None) -> torch.Tensor:
        use64 = (self.precision == "fp64") if fp64 is None else fp64
        c = self.cache
        self.napply += Q.shape[0]
        if use64:
            return self._apply64(k, Q)
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
    """Orthonormal rows spanning R: one Cholesky-QR pass (Gram matrix by GEMM
    in R's precision, Cholesky in FP64, triangular solve in R's precision).
    Rows are normalised first and the Gram matrix gets a shift of 10 u (u =
    unit roundoff of R's type), so that nearly dependent rows still factor;
    callers apply it twice with a re-projection in between (CholQR2)."""
    if R.shape[0] == 0:
        return R
    u = 6e-8 if R.dtype == torch.complex64 else 1.1e-16
    nrm = torch.linalg.vector_norm(R, dim=1)
    R = R / torch.clamp(nrm, min=torch.finfo(nrm.dtype).tiny)[:, None]
    S = (R.conj() @ R.transpose(0, 1)).to(torch.complex128)
    S = 0.5 * (S + S.conj().transpose(0, 1))
    eye = torch.eye(S.shape[0], dtype=S.dtype, device=S.device)
    U, info = torch.linalg.cholesky_ex(S + (10.0 * u) * eye, upper=True)
    if int(info) != 0:
        U = torch.linalg.cholesky(S + (1e5 * u) * eye, upper=True)
    return torch.linalg.solve_triangular(U.transpose(0, 1).to(R.dtype), R, upper=False).contiguous()


def _project_out(R, Q):
    for _ in range(2):
        R = R - (R @ Q.conj().transpose(0, 1)) @ Q
    return R


def _svqb_rows(R: torch.Tensor, drop: float) -> torch.Tensor:
    """Orthonormal rows spanning R by SVQB: eigen-decomposition of the Gram
    matrix of the normalised rows (in R's precision); directions with Gram
    eigenvalue below ``drop`` x the largest are numerically dependent and left
    out, the rest are scaled by w^-1/2."""
    nrm = torch.linalg.vector_norm(R, dim=1)
    R = R / torch.clamp(nrm, min=torch.finfo(nrm.dtype).tiny)[:, None]
    S = R.conj() @ R.transpose(0, 1)
    w, V = torch.linalg.eigh(0.5 * (S + S.conj().transpose(0, 1)))
    keep = w > drop * torch.clamp(w.max(), min=torch.finfo(w.dtype).tiny)
    if not bool(keep.all()):
        w, V = w[keep], V[:, keep]
    return ((V.conj() / torch.sqrt(w)[None, :]).transpose(0, 1) @ R).contiguous()


def _new_block(R: torch.Tensor, Q: torch.Tensor, rel: float = 1e-5) -> torch.Tensor:
    """Orthonormal rows spanning the part of R orthogonal to the orthonormal
    rows Q: CholQR2 with re-projection.  Rows that the projection shrinks below
    ``rel`` of their norm lie numerically in span(Q) and are dropped.  A block
    too ill-conditioned for CholQR2 in its precision (Gram matrix off the
    identity by more than 1e-3 afterwards) is rebuilt by SVQB, which leaves out
    the dependent combinations."""
    n0 = torch.linalg.vector_norm(R, dim=1)
    R = _project_out(R, Q)
    keep = torch.linalg.vector_norm(R, dim=1) > rel * n0
    if not bool(keep.all()):
        R = R[keep]
    if R.shape[0] == 0:
        return R
    B = _orth_rows(_project_out(_orth_rows(R), Q))
    G = B.conj() @ B.transpose(0, 1)
    G.diagonal().sub_(1.0)
    if float(torch.max(torch.abs(G))) > 1e-3:
        B = _orth_rows(_project_out(_svqb_rows(R, 1e-5 if R.dtype == torch.complex64 else 1e-12), Q))
    return B


# FP32 Davidson stops at this residual norm; the FP64-anchored refinement takes over below it.
FP32_EIG_FLOOR = 1e-5
# refinement shape: FP32 blocks per cycle, and the cycle cap per anchor
REFINE_INNER = 2
REFINE_CYCLES = 40


@dataclass
class DavidsonResult:
    eig: torch.Tensor
    vec: torch.Tensor
    resid: float
    iters: int
    anchor: object = None     # refine_lowest: the Anchor for the next potential


def davidson_lowest(H: HApply, k: int, X0: torch.Tensor, nband: int, diag: torch.Tensor, max_sub: int,
                    max_iter: int, tol: float, precond: str = "abacus", weights: torch.Tensor = None):
    """Block Davidson for the lowest nband states of H at k (davidson.py:32-77), rows = vectors.

    Stops when the largest residual norm |H x - lambda x| (times the band's
    weight, when ``weights`` is given) drops below tol.  The
    projected matrix is grown block by block (only the new rows/columns are
    computed), only the nb Ritz vectors are formed each iteration, and the
    subspace restarts from them when it would exceed max_sub.  In FP32 mode the
    subspace and its H image are stored in complex64 (cuBLAS CGEMMs) and the
    Rayleigh-Ritz eigh runs in complex64; the Cholesky factors of the
    orthonormalisation are FP64 in both modes.
    """
    nb = int(nband)
    nG = X0.shape[1]
    max_sub = min(int(max_sub), nG)
    cdt = torch.complex64 if H.precision == "fp32" else torch.complex128
    Q = _orth_rows(X0.to(cdt))
    HQ = H.apply_native(k, Q)
    T = _hermitize((Q.conj() @ HQ.transpose(0, 1)).to(torch.complex128))
    lam, resid, it = None, float("inf"), 0
    X = None
    if cdt == torch.complex64:
        tol = max(tol, FP32_EIG_FLOOR)
    hist = []
    for it in range(1, max_iter + 1):
        # the FP32 phase's Rayleigh-Ritz in complex64 (T is built from complex64 products)
        w, U = torch.linalg.eigh(T.to(cdt))
        w = w.to(torch.float64)
        Ub = U[:, :nb].transpose(0, 1).to(cdt)
        X, HX, lam = Ub @ Q, Ub @ HQ, w[:nb]
        R = HX - lam.to(X.real.dtype)[:, None] * X
        rn = torch.linalg.vector_norm(R, dim=1).to(torch.float64)
        if weights is not None:
            rn = rn * weights
        resid = float(rn.max())
        hist.append(resid)
        if resid < tol or it == max_iter:
            break
        # FP32 rounding floor: near it, stop when six iterations did not halve the residual
        if (cdt == torch.complex64 and resid < 100 * FP32_EIG_FLOOR and len(hist) > 6
                and resid > 0.5 * min(hist[:-6])):
            break
        active = rn > 0.1 * tol
        R = R[active] / _precond(lam[active], diag, precond).to(X.real.dtype)
        if Q.shape[0] + R.shape[0] > max_sub:
            Q, HQ = X, HX
            T = torch.diag(lam).to(torch.complex128)
        # projections in the storage precision, Cholesky factors in FP64
        qadd = _new_block(R, Q)
        if qadd.shape[0] == 0:
            break
        hadd = H.apply_native(k, qadd)
        m = Q.shape[0]
        Q = torch.cat([Q, qadd], 0)
        HQ = torch.cat([HQ, hadd], 0)
        T12 = (Q.conj() @ hadd.transpose(0, 1)).to(torch.complex128)      # (m + kk, kk)
        Tn = torch.empty((Q.shape[0], Q.shape[0]), dtype=torch.complex128, device=Q.device)
        Tn[:m, :m] = T
        Tn[:, m:] = T12
        Tn[m:, :m] = T12[:m].conj().transpose(0, 1)
        T = _hermitize(Tn)
    return DavidsonResult(eig=lam, vec=X.to(torch.complex128).contiguous(), resid=resid, iters=it)


def _ritz_fp64(X, HX):
    """Ritz pairs of the pencil (X^H H X, X^H X) in FP64; returns lambda and the
    rotated rows U^T X, U^T H X (U^H S U = I, U^H T U = diag(lambda))."""
    S = _hermitize(_mm64(X, X.transpose(0, 1), conj_a=True))
    T = _hermitize(_mm64(X, HX.transpose(0, 1), conj_a=True))
    nb = X.shape[0]
    L = torch.linalg.cholesky(S)
    eye = torch.eye(nb, dtype=S.dtype, device=S.device)
    Li = torch.linalg.solve_triangular(L, eye, upper=False)
    w, V = torch.linalg.eigh(_hermitize(Li @ T @ Li.conj().transpose(0, 1)))
    Ut = (Li.conj().transpose(0, 1) @ V).transpose(0, 1)
    Xr, HXr = _rotate(Ut, X, HX)
    return w, Xr, HXr


# relative error of one FP32 H psi: 8 unit roundoffs, the accumulation of a
# radix-8/9/15 FFT chain or a length-n dot product at n ~ 10^2..10^5
FP32_APPLY_ERR = 8 * 6e-8

# The refinement's FP64 subspace products (projections off X, Rayleigh-Ritz at the
# anchors, rotations of X and H X) run in double-float arithmetic on the FP32 pipes
# (ops.zgemm_df, ~1e-14 relative) unless ADDFT_DF_GEMM=0 (cuBLAS ZGEMM, ~1 TFLOP/s on
# GB300).  DF_ERR bounds the relative error one such rotation adds to H X.
DF_GEMM = os.environ.get("ADDFT_DF_GEMM", "1") != "0"
DF_ERR = 3e-14


def _mm64(a, b, conj_a=False, conj_b=False):
    """op(a) @ op(b) for complex128 matrices, to ~1e-14 relative (host tensors, which
    only the host-logic tests with a dense stand-in H use, go through torch)."""
    if DF_GEMM and a.is_cuda:
        return ops.zgemm_df(a, b, conj_a, conj_b)
    return (a.conj() if conj_a else a) @ (b.conj() if conj_b else b)


def _rotate(U, X, HX):
    """U X and U H X (FP64-accurate products)."""
    return _mm64(U, X), _mm64(U, HX)


@dataclass
class Anchor:
    """FP64-accurate H X for orthonormal Ritz vectors X (rows) with Ritz values
    lam, valid for the potential v; ``drift`` estimates (as a bound) the FP32
    rounding that the incremental updates have added to H X since it was last
    computed in FP64: e max|dv| per potential change and
    e max_j sum_b |U_B[j, b]| max_b |H b| per cycle (e = FP32_APPLY_ERR)."""
    X: torch.Tensor
    HX: torch.Tensor
    lam: torch.Tensor
    v: torch.Tensor
    drift: float = 0.0
    Y: torch.Tensor = None    # complex64 buffer states above the window


def refine_lowest(H: HApply, k: int, X: torch.Tensor, nband: int, diag: torch.Tensor, iters: int, tol: float,
                  precond: str = "abacus", verify: bool = False, inner: int = 2, cycles: int = 40,
                  weights: torch.Tensor = None, anchor: Anchor = None, trace: list = None,
                  Y: torch.Tensor = None):
    """FP64-anchored refinement of the lowest Ritz pairs (defect correction).

    Anchor: H X exact to FP64 rounding, either from the FP64 kernels or carried
    over from the previous potential (``anchor``): H' X = H X + (v' - v) X,
    where the FP32 kernels apply the small potential change.  The Ritz pairs
    of X in FP64 then make R = H X - lambda X exact.

    A cycle is a block Davidson on [X, Y, P, C_1, ..., C_m] (m <= ``inner``):
    Y = buffer states above the window (complex64, never anchored), P = the
    previous cycle's step, C_j = K^-1 R_j (preconditioned Ritz residual).
    Each block is orthonormalised in FP32, projected off X in FP64 and kept in
    complex128, so B^H X = 0 to FP64 rounding; H B uses the FP32 kernels.  With
    B orthogonal to X the coupling block is <b|H|x_a> = b^H R_a, a product of
    small quantities, and the X-X block is diag(lambda); only the B-B block
    carries FP32 error.  Rayleigh-Ritz steps inside a cycle run in complex64
    (they only steer the next block,
        R_j = [U_X (lambda_a - lambda_j)] X + U_X R + U_B (H B - lambda_j B));
    the cycle ends with an FP64 eigh of the assembled matrix and
        X <- U_X X + U_B B,   H X <- U_X (H X) + U_B (H B),   R = H X - lambda X
    with the U_X parts in FP64 and the U_B parts in FP32.  U_B is of the size
    of the residual for every band that stays in the window, so FP32 rounding
    enters H X and X in proportion to it; the next Ritz vectors above the
    window become the new Y.

    Cycles run until max |R| < tol (at most ``cycles``).  ``iters`` bounds the
    FP64 anchors; with ``verify`` the final vectors are anchored once more in
    FP64 and the returned residual is exact.  Returns the eigenpairs, the number
    of FP64 H X blocks (``iters``), the Anchor for the next potential and the
    buffer Y (``anchor.Y``).  Residual norms are scaled by ``weights`` as in
    davidson_lowest; ``trace`` (a list) receives (kind, max residual, block
    rows) per anchor and cycle.
    """
    nb = int(nband)
    c64, c128 = torch.complex64, torch.complex128
    lam, resid, n64, drift = None, float("inf"), 0, 0.0
    nY = 0 if Y is None else int(Y.shape[0])

    def wnorm(R):
        rn = torch.linalg.vector_norm(R, dim=1).to(torch.float64)
        return rn * weights if weights is not None else rn

    nanchor = iters + (1 if verify else 0)
    for a in range(nanchor):
        if a == 0 and anchor is not None:
            # carried anchor: H' X = H X + dv X and T = X^H H' X = diag(lam) + X^H (dv X).  X stays
            # unrotated (the first cycle's FP64 eigh absorbs the rotation); the block residual
            # R = H' X - T^T X = (H X - lam X) + dv X - dT^T X is built from small FP32 terms.
            X, lam0 = anchor.X, anchor.lam
            X32 = X.to(c64)
            dv = (H.v64 - anchor.v).to(torch.float32)
            dVX = H.apply_local(k, X32, dv)
            HX = anchor.HX + dVX.to(c128)
            drift = anchor.drift + FP32_APPLY_ERR * float(torch.max(torch.abs(dv)))
            dT = X32.conj() @ dVX.transpose(0, 1)
            dT = 0.5 * (dT + dT.conj().transpose(0, 1))
            Txx = torch.diag(lam0).to(c128) + dT.to(c128)
            R = (anchor.HX - lam0[:, None] * X) + (dVX - dT.transpose(0, 1) @ X32).to(c128)
            lam = torch.diagonal(Txx).real.clone()
        else:
            X = X.to(c128)
            HX = H.apply(k, X, fp64=True)
            n64 += 1
            drift = 0.0
            lam, X, HX = _ritz_fp64(X, HX)
            Txx = torch.diag(lam).to(c128)
            R = HX - lam[:, None] * X
        rn = wnorm(R)
        resid = float(rn.max())
        if trace is not None:
            trace.append(("anchor" if n64 else "carried", resid, 0))
        if resid < tol or a == nanchor - 1 and (verify or a > 0):
            if a == 0 and anchor is not None:
                # converged on the carried anchor: rotate to Ritz pairs (FP64)
                w, V = torch.linalg.eigh(_hermitize(Txx))
                lam = w
                X, HX = _rotate(V.transpose(0, 1), X, HX)
            break
        P = None
        for _ in range(cycles):
            X32, R32 = X.to(c64), R.to(c64)
            Bs, HBs = [], []

            def add_block(B):
                prev = torch.cat([X32] + [b.to(c64) for b in Bs], 0)
                B = _new_block(B, prev)
                B64 = B.to(c128)
                coef = _mm64(B64, X.transpose(0, 1), conj_b=True)   # FP64-accurate, O(FP32 eps)
                # a row whose X part is not at rounding level was not resolved in FP32
                ok = torch.linalg.vector_norm(coef, dim=1) < 1e-5
                if not bool(ok.all()):
                    B64, coef = B64[ok], coef[ok]
                if B64.shape[0] == 0:
                    return
                B64 = B64 - (coef.to(c64) @ X32).to(c128)
                Bs.append(B64)
                HBs.append(H.apply_native(k, B64.to(c64)))

            if Y is not None:
                add_block(Y.to(c64))
            if P is not None:
                # the previous step of the bands that are still unconverged
                keep = (rn > 0.1 * tol) & (torch.linalg.vector_norm(P, dim=1) > 0)
                if bool(keep.any()):
                    add_block(P[keep])
            Ri, lami, rni, Tf = R32, lam, rn, None
            if Bs:
                Tf = _assemble(Txx, R32, Bs, HBs)
            for j in range(inner):
                active = rni > 0.1 * tol
                if not bool(active.any()):
                    break
                nblk = len(Bs)
                add_block(Ri[active] / _precond(lami[active], diag, precond).to(torch.float32))
                if len(Bs) == nblk:
                    break
                Tf = _assemble(Txx, R32, Bs, HBs)
                if j == inner - 1:
                    break
                # steering Rayleigh-Ritz in complex64: it only picks the next block
                B32, HB = torch.cat(Bs, 0).to(c64), torch.cat(HBs, 0)
                w, U = torch.linalg.eigh(Tf.to(c64))
                lami = w[:nb].to(torch.float64)
                Ub32 = U[:, :nb].transpose(0, 1)
                UX32, UB32 = Ub32[:, :nb], Ub32[:, nb:]
                UX = Ub32[:, :nb].to(c128)
                M = (UX @ Txx.conj() - lami[:, None] * UX).to(c64)
                Ri = M @ X32 + UX32 @ R32 + UB32 @ HB - (lami.to(torch.float32)[:, None] * UB32) @ B32
                rni = wnorm(Ri)
                if float(rni.max()) < 0.5 * tol:
                    break
            if Tf is None:
                break
            w, U = torch.linalg.eigh(Tf)
            lam, Ub = w[:nb], U[:, :nb].transpose(0, 1)              # (nb, nb + kb)
            Txx = torch.diag(lam).to(c128)
            B32, HB = torch.cat(Bs, 0).to(c64), torch.cat(HBs, 0)
            UB32 = Ub[:, nb:].to(c64)
            ny = min(nY, U.shape[1] - nb)
            if ny:
                Uy = U[:, nb:nb + ny].transpose(0, 1).to(c64)
                Y = torch.cat([Uy[:, :nb] @ X32 + Uy[:, nb:] @ B32, Y[ny:].to(c64)], 0)
            P = UB32 @ B32
            HP = UB32 @ HB
            Xr, HXr = _rotate(Ub[:, :nb], X, HX)
            X = Xr + P.to(c128)
            HX = HXr + HP.to(c128)
            # FP32 error of H B is ~e |H| per unit block row; U_B weighs it in
            drift += (FP32_APPLY_ERR * float(torch.max(torch.sum(torch.abs(UB32), dim=1)))
                      * float(torch.max(torch.linalg.vector_norm(HB, dim=1))))
            if DF_GEMM and HX.is_cuda:   # the double-float rotation of H X
                drift += DF_ERR * float(torch.max(torch.linalg.vector_norm(HX, dim=1)))
            R = HX - lam[:, None] * X
            rn = wnorm(R)
            resid = float(rn.max())
            if trace is not None:
                trace.append(("cycle", resid, sum(b.shape[0] for b in Bs)))
            if resid < tol:
                break
        if not verify:
            break
    return DavidsonResult(eig=lam, vec=X.contiguous(), resid=resid, iters=n64,
                          anchor=Anchor(X=X, HX=HX, lam=lam, v=H.v64, drift=drift, Y=Y))


def _assemble(Txx, R32, Bs, HBs):
    """Projected matrix on [X, B]: X^H H X | B^H R | B^H H B (FP64 storage)."""
    nb = Txx.shape[0]
    c64, c128 = torch.complex64, torch.complex128
    B32, HB = torch.cat(Bs, 0).to(c64), torch.cat(HBs, 0)
    kb = B32.shape[0]
    Tf = torch.zeros((nb + kb, nb + kb), dtype=c128, device=Txx.device)
    Tf[:nb, :nb] = Txx
    Tbx = (B32.conj() @ R32.transpose(0, 1)).to(c128)
    Tf[nb:, :nb] = Tbx
    Tf[:nb, nb:] = Tbx.conj().transpose(0, 1)
    Tf[nb:, nb:] = (B32.conj() @ HB.transpose(0, 1)).to(c128)
    return _hermitize(Tf)


# ---------------------------------------------------------------------------
# DIIS mixer (mixer.py:23-82), on device tensors
# ---------------------------------------------------------------------------

class _PulayHistory:
    """Last m (rho_in, residual) pairs with their residual Gram matrix, which is
    updated by one matrix-vector product per step; ``coefficients`` solves
    the constrained least-squares problem of Pulay/DIIS (mixer.py:40-70)."""

    def __init__(self, m: int):
        self.m = int(m)
        self.rins, self.res = [], []
        self.G = None

    def reset(self):
        self.rins.clear()
        self.res.clear()
        self.G = None

    def append(self, rho_in, r):
        if len(self.rins) == self.m:
            self.rins.pop(0)
            self.res.pop(0)
            self.G = self.G[1:, 1:]
        g = torch.stack(self.res + [r]) @ r if self.res else (r @ r).reshape(1)
        n = len(self.res) + 1
        G = torch.empty((n, n), dtype=torch.float64, device=r.device)
        if n > 1:
            G[:-1, :-1] = self.G
        G[-1, :] = g
        G[:, -1] = g
        self.G = G
        self.rins.append(rho_in)
        self.res.append(r)

    def coefficients(self):
        n = len(self.res)
        B = torch.zeros((n + 1, n + 1), dtype=torch.float64, device=self.G.device)
        B[:n, :n] = self.G
        B[:n, n] = -1.0
        B[n, :n] = -1.0
        B = B + torch.eye(n + 1, dtype=torch.float64, device=B.device) * 1e-12
        rhs = torch.zeros(n + 1, dtype=torch.float64, device=B.device)
        rhs[n] = -1.0
        return torch.nan_to_num(torch.linalg.solve(B, rhs)[:n], nan=0.0, posinf=0.0, neginf=0.0)


class DIISMixer:
    """Pulay/DIIS, history m = 8, rho_new = sum c_i (rho_in_i + beta r_i), restart on
    non-finite (mixer.py:23-82)."""

    def __init__(self, m: int = 8, beta: float = 0.5):
        self.beta = float(beta)
        self.h = _PulayHistory(m)

    def reset(self):
        self.h.reset()

    def __call__(self, rho_in, rho_out):
        self.h.append(rho_in, rho_out - rho_in)
        if len(self.h.res) == 1:
            return rho_in + self.beta * (rho_out - rho_in)
        c = self.h.coefficients()
        new = c @ (torch.stack(self.h.rins) + self.beta * torch.stack(self.h.res))
        if not bool(torch.isfinite(new).all()):
            self.reset()
            return rho_in + self.beta * (rho_out - rho_in)
        return new


# density residual below which the FP32 SCF hands over to FP64-anchored steps
REFINE_SWITCH = 1e-4
# eigensolver tolerance per SCF step = EIG_TOL_FACTOR x density residual (within [1e-11, 1e-3])
EIG_TOL_FACTOR = 0.3
# FP32 runs take the density band sum in FP32 while the residual is above this
DENSITY_FP32_ABOVE = 1e-4
# the mixer history is dropped when the residual grows by more than this factor
MIX_RESTART_FACTOR = 1.5


class PulayKerkerMixer:
    """Pulay/DIIS on the density residuals with a Kerker-preconditioned step:
    rho_new = sum_i c_i rho_in_i + K(sum_i c_i r_i), K = alpha q^2/(q^2 + gg0)
    (the reference's kerker_mix, scf.py:215-223, applied to the DIIS
    extrapolated residual; history m = 8 and restart rules as mixer.py)."""

    def __init__(self, static: Static, cache: GeometryCache, m: int = 8, alpha: float = 0.7, gg0: float = 0.5):
        self.alpha, self.gg0 = float(alpha), float(gg0)
        self.full = static.device().full
        self.bvec = cache.bvec
        self.h = _PulayHistory(m)

    def reset(self):
        self.h.reset()

    def kerker(self, x):
        return ops.kerker(self.full, self.bvec, x, self.alpha, self.gg0)

    def __call__(self, rho_in, rho_out):
        self.h.append(rho_in, rho_out - rho_in)
        if len(self.h.res) == 1:
            return rho_in + self.kerker(self.h.res[0])
        c = self.h.coefficients()
        new = c @ torch.stack(self.h.rins) + self.kerker(c @ torch.stack(self.h.res))
        if not bool(torch.isfinite(new).all()):
            self.reset()
            return rho_in + self.kerker(rho_out - rho_in)
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
    refine_iters: int = 3
    precond: str = "abacus"


class Eigensolver:
    """Lowest nband Ritz pairs of H[v] per k with warm starts across SCF steps.

    The iterative solvers carry NBUF = max(2, ceil(nband / 20)) buffer bands:
    they take part in every Rayleigh-Ritz step but not in the convergence
    test, so a state that crosses the top of the band window cannot stall it."""

    def __init__(self, static: Static, cache: GeometryCache, opts: EigenOptions):
        self.static, self.cache, self.opts = static, cache, opts
        nG = static.basis.nG
        self.dense = opts.solver == "dense" or (opts.solver == "auto" and nG <= opts.dense_max_nG)
        nb = static.nband
        self.nbx = min(nG, nb + max(2, -(-nb // 20)))
        self.weights = torch.zeros(self.nbx, dtype=torch.float64, device="cuda")
        self.weights[:nb] = 1.0
        self.X = None
        self.anchors = [None] * static.nk     # carried FP64-accurate H X per k (refinement)
        self.napply64 = 0
        self.napply32 = 0

    def _start(self, nG, nb):
        # cold start: the lowest-|G| plane waves (scf.py:359-360)
        X = torch.zeros((self.static.nk, nb, nG), dtype=torch.complex128, device="cuda")
        idx = torch.arange(nb, device="cuda")
        X[:, idx, idx] = 1.0
        return X

    def solve(self, v_eff: torch.Tensor, tol: float, refine: bool = False, final: bool = False):
        st, c, o = self.static, self.cache, self.opts
        nb, nk, nG, nbx = st.nband, st.nk, st.basis.nG, self.nbx
        H = HApply(st, c, v_eff, "fp64" if self.dense else o.precision)
        eig = torch.empty((nk, nb), dtype=torch.float64, device="cuda")
        vec = torch.empty((nk, nb, nG), dtype=torch.complex128, device="cuda")
        resid = 0.0
        if self.X is None and not self.dense:
            self.X = self._start(nG, nbx)
        Xn = None if self.dense else torch.empty_like(self.X)
        for k in range(nk):
            if self.dense:
                w, v, r = dense_lowest(H, k, nb)
                self.napply64 += nG
            else:
                # the reference's max(48, 4 nband) (scf.py:318-320); 2 nband for large band counts,
                # where the cost of the FP64 subspace eigh grows with the cube of its size
                max_sub = o.max_sub or (max(48, 4 * nbx) if nbx < 64 else 2 * nbx)
                diag = c.kin[k] + torch.mean(v_eff)
                if refine and o.precision == "fp32":
                    # carry the FP64 anchor across potentials while its FP32 drift stays
                    # well below the requested residual; the final solve re-anchors.
                    # The buffer bands ride along as the FP32 block Y.
                    anc = self.anchors[k]
                    if final or anc is None or anc.drift > 0.1 * tol:
                        anc = None
                    res = refine_lowest(H, k, self.X[k, :nb], nb, diag, o.refine_iters if final else 1, tol,
                                        o.precond, verify=final, inner=REFINE_INNER, cycles=REFINE_CYCLES,
                                        anchor=anc, Y=self.X[k, nb:].to(torch.complex64) if nbx > nb else None)
                    self.anchors[k] = res.anchor
                    self.napply64 += nb * res.iters
                    H.napply -= nb * res.iters
                    Xn[k, :nb] = res.vec
                    if nbx > nb:
                        Xn[k, nb:] = res.anchor.Y.to(torch.complex128)
                else:
                    self.anchors[k] = None
                    res = davidson_lowest(H, k, self.X[k], nbx, diag, max_sub, o.max_iter, tol, o.precond,
                                          weights=self.weights)
                    Xn[k] = res.vec
                w, v, r = res.eig[:nb], res.vec[:nb], res.resid
            eig[k], vec[k] = w, v
            resid = max(resid, r)
        if not self.dense:
            if o.precision == "fp32":
                self.napply32 += H.napply
            else:
                self.napply64 += H.napply
            self.X = Xn
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
              mixer="auto", beta=0.5, driver="auto", eigh_solver="auto", precision="fp64",
              cache: GeometryCache = None, rho0=None, polish: int = 4, stats: dict = None) -> SCFState:
    """DIIS SCF with 4 unmixed polish steps and a final diagonalisation (scf.py:239-282).

    ``eigh_solver`` in {"auto", "dense", "davidson"}; ``precision`` in {"fp64", "fp32"}.
    ``alpha``, ``gg0``, ``driver`` are accepted for signature parity with the reference.
    """
    del driver
    cache = cache or build_geometry_cache(geo, static)
    opts = EigenOptions(solver=eigh_solver, precision=precision)
    eigs = Eigensolver(static, cache, opts)
    rho = initial_density(static, cache) if rho0 is None else rho0
    if mixer == "auto":
        # the reference moves larger cells off plain DIIS onto Kerker (scf.py:571-581)
        mixer = "diis" if (static.natom <= 2 or static.basis.nG <= 800) else "pulay-kerker"
    if mixer == "diis":
        mix = DIISMixer(m=8, beta=beta)
    elif mixer == "pulay-kerker":
        mix = PulayKerkerMixer(static, cache, m=8, alpha=0.7 if alpha == 0.9 else alpha, gg0=gg0)
    else:
        raise ValueError(f"unknown mixer {mixer!r} (diis | pulay-kerker | auto)")
    prev, res, it = 1e9, 1.0, 0
    fp32 = precision == "fp32" and not eigs.dense
    refine, hist = False, []
    for it in range(1, max_iter + 1):
        tol_eig = max(min(1e-3, EIG_TOL_FACTOR * res), 1e-11)
        # FP32 phase until the density residual reaches the FP32 regime (or stops
        # falling), then every step is anchored on FP64 H psi
        refine = fp32 and (refine or res < REFINE_SWITCH
                           or (len(hist) >= 4 and res > 0.5 * min(hist[:-3])))
        v_eff, _ = effective_potential(static, cache, rho)
        eig, psi, eres = eigs.solve(v_eff, tol_eig, refine=refine)
        occ, mu = occupations(static, eig)
        # FP32 band sum while its ~1e-7 error is far below the residual
        rho_out = density_of(static, cache, psi, occ, fp32=fp32 and res > DENSITY_FP32_ABOVE)
        res = float(density_residual(static, cache, rho_out, rho))
        hist.append(res)
        if res > prev * MIX_RESTART_FACTOR:
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
    eig, psi, eres = eigs.solve(v_eff, 1e-11, refine=fp32, final=True)
    occ, mu = occupations(static, eig)
    if stats is not None:
        stats.update(napply64=eigs.napply64, napply32=eigs.napply32, iters=it, eig_resid=eres)
    return SCFState(psi=psi, eig=eig, occ=occ, mu=mu, rho_r=rho, n_iter=it, residual=res)
