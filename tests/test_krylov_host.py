"""The BiCGSTAB of the fixed-point adjoint (response.bicgstab, restating diff/implicit.py:53-65) on
the host, no GPU: a nonsymmetric system of the adjoint's shape, (I - J^T) lam = g with J a
contraction, against a direct solve; a zero right-hand side (a loss that does not depend on the
density) gives lam = 0 at once, as the reference's solver does; a breakdown returns instead of
dividing by zero, and the adjoint's residual check then reports it.  The adjoint solve itself
(response._solve_adjoint) runs on a stand-in exposing only the transposed apply: its matrix-free
and dense modes agree, and a non-convergent solve raises RuntimeError (a host-side fault test:
a BiCGSTAB that fails to converge)."""

from __future__ import annotations

import numpy as np
import torch

from addft_gb300.response import bicgstab


def _system(n, seed=0):
    rng = np.random.default_rng(seed)
    j = rng.normal(size=(n, n))
    j *= 0.7 / np.max(np.abs(np.linalg.eigvals(j)))          # spectral radius 0.7, nonsymmetric
    a = np.eye(n) - j.T
    return torch.as_tensor(a), torch.as_tensor(rng.normal(size=n))


def test_bicgstab_solves_the_adjoint_shaped_system():
    a, g = _system(200)
    lam, nit = bicgstab(lambda y: a @ y, g, rtol=1e-12)
    ref = torch.linalg.solve(a, g)
    assert float(torch.linalg.vector_norm(lam - ref) / torch.linalg.vector_norm(ref)) < 1e-10
    assert 1 <= nit < 200


def test_bicgstab_zero_right_hand_side_returns_zero():
    a, g = _system(50, seed=1)
    lam, nit = bicgstab(lambda y: a @ y, torch.zeros_like(g))
    assert nit == 0 and torch.count_nonzero(lam) == 0


def test_bicgstab_exact_in_one_step_and_breakdown_does_not_divide_by_zero():
    g = torch.arange(1.0, 9.0, dtype=torch.float64)
    lam, nit = bicgstab(lambda y: 3.0 * y, g)                  # a multiple of I: exact after one step
    assert nit == 1 and torch.allclose(lam, g / 3.0, rtol=0, atol=1e-15)
    rot = torch.tensor([[0.0, -1.0], [1.0, 0.0]], dtype=torch.float64)
    lam, nit = bicgstab(lambda y: rot @ y, torch.tensor([1.0, 0.0], dtype=torch.float64))
    assert torch.all(torch.isfinite(lam))                      # <rhat, A r> = 0: stops, no exception


class _StandInResponse:
    """What the adjoint solve uses of a Response: the transposed apply y -> J^T y."""

    def __init__(self, j):
        self.j = j

    def apply_t(self, y):
        return self.j.T @ y


def test_adjoint_solve_modes_agree_and_non_convergence_is_reported():
    """(I - J^T) lam = g through response._solve_adjoint: the matrix-free BiCGSTAB and the dense
    assembly agree; a singular system (J = I) is reported by the residual check as the
    reference's implicit.py:62-65 does (RuntimeError), not by an arithmetic exception; the dense
    form refuses boxes above its size limit."""
    import pytest
    from addft_gb300 import response as R
    a, g = _system(60, seed=2)
    resp = _StandInResponse(torch.eye(60, dtype=torch.float64) - a.T)      # I - J^T = a
    lam_mf, _, res_mf = R._solve_adjoint(resp, g, "matrix_free", 1e-12)
    lam_d, _, res_d = R._solve_adjoint(resp, g, "dense", 1e-12)
    assert res_mf < 1e-10 and res_d < 1e-12
    assert float(torch.linalg.vector_norm(lam_mf - lam_d) / torch.linalg.vector_norm(lam_d)) < 1e-9
    with pytest.raises(RuntimeError, match="did not converge"):
        R._solve_adjoint(_StandInResponse(torch.eye(20, dtype=torch.float64)), torch.ones(20, dtype=torch.float64),
                         "matrix_free", 1e-10)
    big = R.DENSE_MAX_NFFT + 1
    with pytest.raises(ValueError, match="limited"):
        R._solve_adjoint(resp, torch.ones(big, dtype=torch.float64), "dense", 1e-10)
