"""Per-kernel differentiation: one ``torch.autograd.Function`` per C-ABI kernel.

The reference gives its native kernels hand-written derivatives behind JAX
custom rules -- the fused XC handler a custom_vjp whose backward multiplies by
the XC kernel f_xc (``physics/xc.py:195-212``), the sphere scatter / gather a
custom_jvp whose transpose is the other one (``kernels/pack.py:151-192``) -- and
lets ``jax.grad`` derive the rest (``ops/hpsi.py``, ``physics/density.py``,
``physics/hartree.py``).  Here every forward and every backward is a call into
libaddft_gb300.so; torch only records the graph:

=================  ==============================  ===========================================
function           forward kernel                  backward kernel(s)
=================  ==============================  ===========================================
``vxc``            addft_xc_lda                    addft_xc_lda_vjp (f_xc g)
``scatter``        addft_ffi_scatter               addft_ffi_gather
``gather``         addft_ffi_gather                addft_ffi_scatter
``psi_to_real``    addft_psi_to_real               addft_real_to_psi x N / Omega
``real_to_psi``    addft_real_to_psi               addft_psi_to_real x Omega / N
``hpsi``           addft_hpsi                      psi: addft_hpsi (H is Hermitian);
                                                   v: addft_density of psi +/- g (polarisation)
``density``        addft_density                   addft_hpsi with V = g, T = 0, no V_NL
``hartree``        addft_hartree                   addft_hartree (the Coulomb kernel is symmetric)
=================  ==============================  ===========================================

Complex tensors follow torch's convention: the gradient of a real loss L with
respect to z is dL/dRe z + i dL/dIm z, so a C-linear map y = M x has the
backward M^H g.
"""

from __future__ import annotations

import torch

from . import ops
from .ops import Plan


class _Vxc(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho):
        v, _, _ = ops.xc_lda(rho.detach())
        ctx.save_for_backward(rho)
        return v

    @staticmethod
    def backward(ctx, g):
        rho, = ctx.saved_tensors
        return ops.xc_lda_vjp(rho.detach(), g.contiguous())


def vxc(rho: torch.Tensor) -> torch.Tensor:
    """v_xc(r) = d(n eps_xc)/dn (PZ81); backward f_xc(rho) g."""
    return _Vxc.apply(rho)


class _Scatter(torch.autograd.Function):
    @staticmethod
    def forward(ctx, c, idx, nfft):
        ctx.idx, ctx.nG = idx, c.shape[-1]
        return ops.ffi_scatter(c.detach(), idx, nfft)

    @staticmethod
    def backward(ctx, g):
        return ops.ffi_gather(g.contiguous(), ctx.idx, ctx.nG), None, None


class _Gather(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid, idx, nG):
        ctx.idx, ctx.nfft = idx, grid.shape[-1]
        return ops.ffi_gather(grid.detach(), idx, nG)

    @staticmethod
    def backward(ctx, g):
        return ops.ffi_scatter(g.contiguous(), ctx.idx, ctx.nfft), None, None


def scatter(c: torch.Tensor, idx: torch.Tensor, nfft: int) -> torch.Tensor:
    """Sphere coefficients (..., nG) into a zeroed flat box (..., nfft); backward = gather."""
    return _Scatter.apply(c, idx, int(nfft))


def gather(grid: torch.Tensor, idx: torch.Tensor, nG: int) -> torch.Tensor:
    """Flat box (..., nfft) onto the sphere (..., nG); backward = scatter."""
    return _Gather.apply(grid, idx, int(nG))


class _PsiToReal(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi, plan, omega):
        ctx.plan, ctx.omega = plan, omega
        return ops.psi_to_real(plan, psi.detach(), omega)

    @staticmethod
    def backward(ctx, g):
        # psi(r) = Omega^-1/2 sum_G c_G e^{iGr}; its adjoint is N/Omega times real_to_psi
        out = ops.real_to_psi(ctx.plan, g.contiguous(), ctx.omega)
        return out * (ctx.plan.N / ctx.omega), None, None


class _RealToPsi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi_r, plan, omega):
        ctx.plan, ctx.omega = plan, omega
        return ops.real_to_psi(plan, psi_r.detach(), omega)

    @staticmethod
    def backward(ctx, g):
        # c_G = Omega^1/2 / N sum_r e^{-iGr} psi(r); its adjoint is Omega/N times psi_to_real
        out = ops.psi_to_real(ctx.plan, g.contiguous(), ctx.omega)
        return out * (ctx.omega / ctx.plan.N), None, None


def psi_to_real(plan: Plan, psi: torch.Tensor, omega: float) -> torch.Tensor:
    return _PsiToReal.apply(psi, plan, float(omega))


def real_to_psi(plan: Plan, psi_r: torch.Tensor, omega: float) -> torch.Tensor:
    return _RealToPsi.apply(psi_r, plan, float(omega))


def _cross_density(plan: Plan, a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """sum over bands and k of Re(conj(a(r)) b(r)), by polarisation through the density kernel:
    |a + b|^2 - |a - b|^2 = 4 Re(conj(a) b); the Omega of both density calls cancels."""
    nk, nb = a.shape[0], a.shape[1]
    ones = torch.ones((nk, nb), dtype=torch.float64, device=a.device)
    plus = ops.density(plan, (a + b).contiguous(), ones, 1.0)
    minus = ops.density(plan, (a - b).contiguous(), ones, 1.0)
    return 0.25 * (plus - minus)


class _Hpsi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi, v_r, plan, kin, proj, dion, omega):
        ctx.plan, ctx.kin, ctx.proj, ctx.dion, ctx.omega = plan, kin, proj, dion, omega
        ctx.save_for_backward(psi, v_r)
        return ops.hpsi(plan, psi.detach(), kin, v_r.detach(), proj, dion)

    @staticmethod
    def backward(ctx, g):
        psi, v_r = ctx.saved_tensors
        g = g.contiguous()
        gpsi = gv = None
        if ctx.needs_input_grad[0]:
            gpsi = ops.hpsi(ctx.plan, g, ctx.kin, v_r.detach(), ctx.proj, ctx.dion)
        if ctx.needs_input_grad[1]:
            # y_G = Omega^1/2 / N sum_r e^{-iGr} v(r) psi(r)  =>  dL/dv(r) = Omega/N Re(conj(g(r)) psi(r))
            # with g(r), psi(r) the Omega^-1/2-normalised real-space fields; the density kernel
            # (called with omega = 1) returns |sum_G c_G e^{iGr}|^2, i.e. Omega |psi(r)|^2.
            gv = _cross_density(ctx.plan, g, psi.detach()) * (1.0 / ctx.plan.N)
            gv = gv.to(v_r.dtype)
        return gpsi, gv, None, None, None, None, None


def hpsi(plan: Plan, psi: torch.Tensor, kin: torch.Tensor, v_r: torch.Tensor, proj=None, dion=None,
         omega: float = 1.0) -> torch.Tensor:
    """(T + V(r) + V_NL) psi, differentiable in psi and v_r (kinetic and projector tables fixed)."""
    return _Hpsi.apply(psi, v_r, plan, kin, proj, dion, float(omega))


class _Density(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi, plan, wocc, omega):
        ctx.plan, ctx.wocc, ctx.omega = plan, wocc, omega
        ctx.save_for_backward(psi)
        return ops.density(plan, psi.detach(), wocc, omega)

    @staticmethod
    def backward(ctx, g):
        psi, = ctx.saved_tensors
        # dL/dc_{b,G} = 2 w_b Omega^-1/2 sum_r e^{-iGr} g(r) psi_b(r) = 2 w_b N / Omega (V_g psi_b)_G,
        # V_g psi the local H psi with potential g, no kinetic or nonlocal term
        nk, nb, nG = psi.shape
        rdt = torch.float64 if psi.dtype == torch.complex128 else torch.float32
        zero_kin = torch.zeros((nk, nG), dtype=rdt, device=psi.device)
        y = ops.hpsi(ctx.plan, psi.detach(), zero_kin, g.contiguous().to(rdt))
        w = ctx.wocc.to(device=psi.device, dtype=rdt).reshape(nk, nb, 1)
        return y * (2.0 * ctx.plan.N / ctx.omega) * w, None, None, None


def density(plan: Plan, psi: torch.Tensor, wocc: torch.Tensor, omega: float) -> torch.Tensor:
    """rho(r) = sum_{k,b} wocc |psi(r)|^2, differentiable in psi."""
    return _Density.apply(psi, plan, wocc, float(omega))


class _Hartree(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, plan, bvec, omega):
        ctx.plan, ctx.bvec, ctx.omega = plan, bvec, omega
        v, _ = ops.hartree(plan, bvec, omega, rho.detach())
        return v

    @staticmethod
    def backward(ctx, g):
        v, _ = ops.hartree(ctx.plan, ctx.bvec, ctx.omega, g.contiguous())
        return v, None, None, None


def hartree(plan: Plan, bvec, omega: float, rho: torch.Tensor) -> torch.Tensor:
    """v_H(r) of rho on the plan's shell, differentiable in rho (the map is symmetric)."""
    return _Hartree.apply(rho, plan, bvec, float(omega))
