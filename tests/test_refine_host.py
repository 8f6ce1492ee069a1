"""FP64-anchored refinement on the host: a dense plane-wave-like Hermitian
operator (growing diagonal + smooth coupling, exact triplets at the bottom)
stands in for H psi.  The "FP32 kernels" apply a complex64 copy of the matrix
in complex64 arithmetic; the anchor applies the complex128 matrix.

Checks: FP32 Davidson alone stalls near its rounding floor; the refinement
reaches FP64-level residuals and eigenvalues, and tracks a run whose
correction applies are exact (so FP32 rounding is not what limits it).
"""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from addft_gb300 import solver  # noqa: E402

N, NB, NOCC = 400, 20, 14


def _operator():
    rng = np.random.default_rng(1)
    kin = np.sort(0.5 * (rng.random(N) * 4.0) ** 2)
    kin[:30] = np.repeat(kin[0:30:3], 3)
    V = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    V = 0.5 * (V + V.conj().T) * 0.02 * np.exp(-0.05 * np.abs(np.subtract.outer(np.arange(N), np.arange(N))))
    H = np.diag(kin) + V - 0.5
    return 0.5 * (H + H.conj().T)


class _DenseH:
    """H = H0 + diag(v): v plays the local potential (diagonal in this basis)."""

    def __init__(self, H, exact32=False, v=None):
        self.v64 = torch.zeros(H.shape[0], dtype=torch.float64) if v is None else v
        self.H64 = torch.tensor(H) + torch.diag(self.v64).to(torch.complex128)
        self.H32 = self.H64.to(torch.complex64)
        self.exact32 = exact32
        self.precision = "fp32"
        self.napply = 0

    def apply(self, k, X, fp64=None):
        self.napply += X.shape[0]
        return X.to(torch.complex128) @ self.H64.T

    def apply_local(self, k, Q, dv):
        self.napply += Q.shape[0]
        return Q * dv.to(torch.float32)[None, :]

    def apply_native(self, k, Q):
        self.napply += Q.shape[0]
        if self.exact32 or Q.dtype == torch.complex128:
            return (Q.to(torch.complex128) @ self.H64.T).to(Q.dtype)
        return Q @ self.H32.T


def test_refinement_reaches_fp64_and_tracks_exact_applies():
    Hm = _operator()
    ev = np.linalg.eigvalsh(Hm)
    W = torch.ones(NB, dtype=torch.float64)
    W[NOCC:] = 1e-4
    diag = torch.tensor(np.real(np.diag(Hm)))
    X0 = torch.zeros((NB, N), dtype=torch.complex128)
    X0[torch.arange(NB), torch.arange(NB)] = 1.0
    H = _DenseH(Hm)
    d = solver.davidson_lowest(H, 0, X0, NB, diag, 80, 80, 1e-12, weights=W)
    assert d.resid > 1e-7                                     # FP32 alone
    r = solver.refine_lowest(H, 0, d.vec, NB, diag, 4, 1e-10, verify=True, inner=2, weights=W)
    r_exact = solver.refine_lowest(_DenseH(Hm, exact32=True), 0, d.vec, NB, diag, 4, 1e-10, verify=True,
                                   inner=2, weights=W)
    assert r.resid < 1e-10 and r_exact.resid < 1e-10
    assert r.iters <= r_exact.iters + 1
    assert np.max(np.abs(r.eig[:NOCC].numpy() - ev[:NOCC])) < 1e-11
    S = r.vec.conj() @ r.vec.T
    assert torch.max(torch.abs(S - torch.eye(NB, dtype=S.dtype))).item() < 1e-12


def test_carried_anchor_follows_a_potential_change_without_fp64_applies():
    """After an FP64 anchor at v1, the next solve at v2 = v1 + dv (dv ~ 1e-4)
    carries H X over with FP32 applies of dv only, and the verified result
    matches the exact eigenvalues of H0 + diag(v2)."""
    Hm = _operator()
    rng = np.random.default_rng(7)
    v1 = torch.zeros(N, dtype=torch.float64)
    v2 = torch.tensor(1e-4 * rng.normal(size=N))
    diag = torch.tensor(np.real(np.diag(Hm)))
    X0 = torch.zeros((NB, N), dtype=torch.complex128)
    X0[torch.arange(NB), torch.arange(NB)] = 1.0
    W = torch.ones(NB, dtype=torch.float64)
    W[NOCC:] = 1e-4
    H1 = _DenseH(Hm, v=v1)
    d = solver.davidson_lowest(H1, 0, X0, NB, diag, 80, 80, 1e-12, weights=W)
    r1 = solver.refine_lowest(H1, 0, d.vec, NB, diag, 4, 1e-10, verify=True, weights=W)
    assert r1.resid < 1e-10
    H2 = _DenseH(Hm, v=v2)
    r2 = solver.refine_lowest(H2, 0, r1.vec, NB, diag, 1, 1e-9, weights=W, anchor=r1.anchor)
    assert r2.iters == 0                       # no FP64 H X: the anchor was carried
    assert r2.resid < 1e-9 and r2.anchor.drift < 1e-7
    ev2 = np.linalg.eigvalsh(H2.H64.numpy())
    assert np.max(np.abs(r2.eig[:NOCC].numpy() - ev2[:NOCC])) < 1e-10   # bounded by the drift
    # the carried residual is the true one to within the drift bound
    R = r2.vec @ H2.H64.T - r2.eig[:, None] * r2.vec
    true = (torch.linalg.vector_norm(R, dim=1) * W).max().item()
    assert abs(true - r2.resid) <= r2.anchor.drift
    HXerr = torch.max(torch.linalg.vector_norm(r2.anchor.HX - r2.anchor.X @ H2.H64.T, dim=1)).item()
    assert HXerr <= r2.anchor.drift
