"""Per-kernel torch.autograd.Function wrappers over the C ABI (addft_gb300.autograd).

Each wrapper's backward is a kernel call of its own (listed in the module); torch's
gradcheck compares it with central differences of the forward kernel in FP64 on the
reference's fixture cell (9^3 box, nG 27) -- the same role the reference gives
jax.test_util.check_grads for its custom_vjp / custom_jvp rules (physics/xc.py:195-212,
kernels/pack.py:151-192).  Tolerance: gradcheck's atol 1e-7 / rtol 1e-5 at eps 1e-6.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import LATTICE, FRAC_DISTORTED, gpu_available

pytestmark = pytest.mark.gpu
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import torch  # noqa: E402

import addft_gb300 as ad  # noqa: E402
from addft_gb300 import autograd as AG  # noqa: E402
from addft_gb300.system import build_geometry_cache  # noqa: E402
from oracle import pw  # noqa: E402

GC = dict(eps=1e-6, atol=1e-7, rtol=1e-5)


@pytest.fixture(scope="module")
def fx():
    s = ad.setup(LATTICE, FRAC_DISTORTED, ecut=2.0, nband=2, density_factor=4.0, sigma=0.05)
    cache = build_geometry_cache(s.geo, s.static)
    plan = s.static.device().wfc
    return s, cache, plan


def _psi(nk, nb, nG, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(nk, nb, nG)) + 1j * rng.normal(size=(nk, nb, nG))
    return torch.as_tensor(x, device="cuda")


def test_vxc_backward_is_fxc_and_passes_gradcheck():
    rng = np.random.default_rng(1)
    rho = torch.as_tensor(rng.uniform(0.01, 0.2, 64), device="cuda").requires_grad_(True)
    assert torch.autograd.gradcheck(AG.vxc, (rho,), **GC)
    g = torch.as_tensor(rng.normal(size=64), device="cuda")
    (gr,) = torch.autograd.grad(AG.vxc(rho), rho, g)
    ref = pw.xc_kernel_point(rho.detach().cpu().numpy()) * g.cpu().numpy()
    assert np.max(np.abs(gr.cpu().numpy() - ref)) < 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("dtype", [torch.complex128])
def test_scatter_gather_backward_are_each_other(fx, dtype):
    s, cache, plan = fx
    idx = torch.as_tensor(pw.flat_index(s.static.basis.fft_shape, s.static.basis.miller), device="cuda")
    N = plan.N
    c = _psi(1, 2, plan.nG, 3)[0].to(dtype).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: AG.scatter(x, idx, N), (c,), **GC)
    grid = _psi(1, 2, N, 4)[0].to(dtype).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: AG.gather(x, idx, plan.nG), (grid,), **GC)


def test_transforms_backward_are_the_adjoints(fx):
    s, cache, plan = fx
    om = cache.omega
    psi = _psi(1, 2, plan.nG, 5)[0].requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: AG.psi_to_real(plan, x, om), (psi,), **GC)
    r = _psi(1, 1, plan.N, 6)[0].requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: AG.real_to_psi(plan, x, om), (r,), **GC)


def test_hpsi_backward_in_psi_and_potential(fx):
    s, cache, plan = fx
    rng = np.random.default_rng(8)
    psi = _psi(1, 2, plan.nG, 7).requires_grad_(True)
    v = torch.as_tensor(rng.uniform(-0.5, 0.5, plan.N), device="cuda").requires_grad_(True)
    f = lambda x, y: AG.hpsi(plan, x, cache.kin, y, cache.proj, cache.dion)  # noqa: E731
    assert torch.autograd.gradcheck(f, (psi, v), **GC)


def test_density_backward_passes_gradcheck(fx):
    s, cache, plan = fx
    psi = _psi(1, 2, plan.nG, 9).requires_grad_(True)
    wocc = torch.tensor([[2.0, 0.7]], dtype=torch.float64, device="cuda")
    assert torch.autograd.gradcheck(lambda x: AG.density(plan, x, wocc, cache.omega), (psi,), **GC)


def test_hartree_backward_passes_gradcheck(fx):
    s, cache, plan = fx
    rng = np.random.default_rng(10)
    rho = torch.as_tensor(rng.uniform(0.0, 0.1, plan.N), device="cuda").requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: AG.hartree(plan, cache.bvec, cache.omega, x), (rho,), **GC)


def test_chain_through_every_kernel_matches_oracle_energy_gradient(fx):
    """E_H + E_xc of rho[psi] differentiated through density -> hartree / vxc backwards, against
    central differences of the same chain on the oracle."""
    s, cache, plan = fx
    om, N = cache.omega, plan.N
    psi = _psi(1, 2, plan.nG, 12) * 0.05
    psi.requires_grad_(True)
    wocc = torch.tensor([[2.0, 2.0]], dtype=torch.float64, device="cuda")
    rho = AG.density(plan, psi, wocc, om)
    vh = AG.hartree(plan, cache.bvec, om, rho)
    loss = 0.5 * (om / N) * torch.sum(vh * rho) + (om / N) * torch.sum(AG.vxc(rho) * rho)
    (g,) = torch.autograd.grad(loss, psi)
    g = g.cpu().numpy()
    o = pw.setup(LATTICE, FRAC_DISTORTED, ecut=2.0, nband=2, density_factor=4.0, sigma=0.05)
    b = o.static.basis

    def oracle_loss(c):
        r = pw.density_from_psi(b, o.lattice, c[None], np.ones((1, 2)), np.ones(1), spin_degeneracy=2.0)
        return (pw.hartree_energy(b, o.lattice, r)
                + (pw.volume(o.lattice) / b.nfft) * np.sum(pw.xc_potential_point(r) * r))

    c0 = psi.detach().cpu().numpy()[0]
    h = 1e-6
    for (bb, G) in [(0, 0), (1, 5), (0, 17)]:
        for part, unit in (("re", 1.0), ("im", 1j)):
            cp, cm = c0.copy(), c0.copy()
            cp[bb, G] += h * unit
            cm[bb, G] -= h * unit
            fd = (oracle_loss(cp) - oracle_loss(cm)) / (2 * h)
            an = g[0, bb, G].real if part == "re" else g[0, bb, G].imag
            assert abs(an - fd) < 1e-6 * max(1.0, abs(fd)), (bb, G, part, an, fd)
