"""The SCF's Pulay/DIIS density mixer on the host (no GPU): solver.DIISMixer, which keeps the
residual Gram matrix updated by one product per step, against the oracle's DIISMixer, which
rebuilds it every step (both restating mixer.py:23-82), on the same sequence of densities.

* a linear contraction map n -> A n + b over more steps than the history holds (m = 8, so the
  oldest pair is evicted): every mixed density agrees to rounding and both reach the fixed point;
* a non-finite extrapolation restarts the history with a plain linear step, as the reference does.
"""

from __future__ import annotations

import numpy as np
import torch

from addft_gb300 import solver
from oracle import pw


def _contraction(n, rho, seed=0):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    a = (q * rng.uniform(-rho, rho, n)) @ q.T          # symmetric, spectral radius < rho
    b = rng.normal(size=n)
    return a, b, np.linalg.solve(np.eye(n) - a, b)


def test_diis_matches_oracle_step_by_step_and_reaches_the_fixed_point():
    n = 64
    a, b, fixed = _contraction(n, 0.6)
    mine, ref = solver.DIISMixer(m=8, beta=0.5), pw.DIISMixer(m=8, beta=0.5)
    x_mine = x_ref = np.zeros(n)
    for step in range(40):
        out_mine = torch.as_tensor(x_mine) @ torch.as_tensor(a).T + torch.as_tensor(b)
        new_mine = mine(torch.as_tensor(x_mine), out_mine).numpy()
        new_ref = ref(x_ref, a @ x_ref + b)
        scale = max(1.0, float(np.max(np.abs(new_ref))))
        assert np.max(np.abs(new_mine - new_ref)) < 1e-9 * scale, step
        x_mine, x_ref = new_mine, new_ref
    assert len(mine.h.res) == 8                          # history capped at m
    assert np.max(np.abs(x_mine - fixed)) < 1e-6 * np.max(np.abs(fixed))   # 3e-8 after 40 steps
    assert np.max(np.abs(x_ref - fixed)) < 1e-6 * np.max(np.abs(fixed))


def test_diis_restarts_on_a_non_finite_extrapolation():
    n = 16
    a, b, _ = _contraction(n, 0.5, seed=1)
    mine, ref = solver.DIISMixer(m=8, beta=0.5), pw.DIISMixer(m=8, beta=0.5)
    x = np.zeros(n)
    for _ in range(3):
        x_next = mine(torch.as_tensor(x), torch.as_tensor(a @ x + b)).numpy()
        ref(x, a @ x + b)
        x = x_next
    out = a @ x + b
    out[0] = np.inf                                      # a non-finite output density
    got = mine(torch.as_tensor(x), torch.as_tensor(out)).numpy()
    want = ref(x, out)
    assert len(mine.h.res) == 0 and len(ref.rins) == 0   # history dropped by both
    lin = x + 0.5 * (out - x)                            # the plain linear step
    assert np.array_equal(got, lin) and np.array_equal(want, lin)
