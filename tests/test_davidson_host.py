"""Block Davidson (solver.davidson_lowest, restating solver/davidson.py:32-77) on the host, no GPU,
with a dense FP64 stand-in for H psi.  The reference checks Davidson against the dense lowest
eigenpairs (tests/test_davidson.py:16-30); here also the cases a production SCF meets:

* exactly degenerate levels straddling the band window (every level threefold: with 8 bands the
  window cuts a triplet in two);
* a start block with linearly dependent rows (the Cholesky-QR / SVQB orthonormalisation);
* one band, and a subspace limit small enough to force restarts.
Eigenvalues within 1e-10 of numpy.linalg.eigvalsh, residual below the tolerance.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from addft_gb300 import solver


class _Dense:
    precision = "fp64"

    def __init__(self, H):
        self.H = torch.as_tensor(H)

    def apply_native(self, k, Q):
        return (Q.to(torch.complex128) @ self.H.T).to(Q.dtype)


def _plane_wave_like(n, seed):
    """Diagonally dominant Hermitian H: levels 0.05 apart on the diagonal (the kinetic term) and a
    smooth random coupling (the potential), so the gaps at the band window are clear."""
    rng = np.random.default_rng(seed)
    kin = 0.05 * np.arange(n) - 0.5
    v = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    v = 0.5 * (v + v.conj().T) * 0.03 * np.exp(-0.05 * np.abs(np.subtract.outer(np.arange(n), np.arange(n))))
    h = np.diag(kin) + v
    return 0.5 * (h + h.conj().T)


def _run(H, nb, X0, max_sub=80, tol=1e-11):
    diag = torch.as_tensor(np.real(np.diag(H)).copy())
    d = solver.davidson_lowest(_Dense(H), 0, X0, nb, diag, max_sub, 300, tol)
    ev = np.linalg.eigvalsh(H)[:nb]
    assert d.resid < tol, d.resid
    assert np.max(np.abs(d.eig.numpy() - ev)) < 1e-10, (d.eig.numpy() - ev)
    X = d.vec
    assert torch.allclose(X.conj() @ X.T, torch.eye(nb, dtype=torch.complex128), atol=1e-10)
    return d


def _unit_rows(nb, n):
    X0 = torch.zeros((nb, n), dtype=torch.complex128)
    X0[torch.arange(nb), torch.arange(nb)] = 1.0
    return X0


def test_threefold_levels_cut_by_the_band_window():
    h = _plane_wave_like(100, seed=3)
    H = np.kron(np.eye(3), h)                     # every level exactly threefold
    ev = np.linalg.eigvalsh(H)
    assert abs(ev[7] - ev[8]) < 1e-12             # the 8-band window cuts a triplet
    rng = np.random.default_rng(4)
    X0 = torch.as_tensor(rng.normal(size=(8, 300)) + 1j * rng.normal(size=(8, 300)))
    _run(H, 8, X0)


def test_linearly_dependent_start_block():
    H = _plane_wave_like(240, seed=5)
    X0 = _unit_rows(10, 240)
    X0[9] = X0[0] + 1e-14 * X0[1]                 # row 9 repeats row 0 to rounding
    X0[8] = 2.0 * X0[3]
    _run(H, 10, X0)


@pytest.mark.parametrize("nb,max_sub", [(1, 80), (12, 26)])
def test_one_band_and_forced_restarts(nb, max_sub):
    H = _plane_wave_like(260, seed=6)
    _run(H, nb, _unit_rows(nb, 260), max_sub=max_sub)
