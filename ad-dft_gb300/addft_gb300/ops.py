"""Thin torch wrappers over the C ABI (device pointers + the current CUDA stream).

Every function here launches GB300 kernels from libaddft_gb300.so through
ctypes; torch only owns the device memory and the stream.  Shapes follow the
reference: psi (nk, nb, nG) complex, real-space fields (N,) with flat index
(i1*n2 + i2)*n3 + i3.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import LIB, check

F32, F64 = _lib.F32, _lib.F64


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("addft_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU path")


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def _dt(t: torch.Tensor) -> int:
    if t.dtype in (torch.complex128, torch.float64):
        return F64
    if t.dtype in (torch.complex64, torch.float32):
        return F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def _c(t: torch.Tensor, what: str) -> torch.Tensor:
    if not t.is_cuda:
        raise ValueError(f"{what} must be a CUDA tensor")
    return t.contiguous()


def _d3(x):
    return _lib.dbl_array(np.asarray(x, dtype=np.float64).reshape(-1))


class _Workspace:
    """Grow-only scratch arena on the current device (torch allocations are 512-B aligned)."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes: int) -> torch.Tensor:
        nbytes = max(int(nbytes), 256)
        if self.buf is None or self.buf.numel() < nbytes or self.buf.device != torch.device("cuda", torch.cuda.current_device()):
            self.buf = None
            self.buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        return self.buf


_WS = _Workspace()


def workspace(nbytes: int) -> torch.Tensor:
    return _WS.get(nbytes)


class Plan:
    """addft_plan: FFT box + frozen G-sphere (host Miller indices)."""

    def __init__(self, fft_shape, miller):
        require_cuda()
        m = np.ascontiguousarray(np.asarray(miller, dtype=np.int32).reshape(-1, 3))
        n1, n2, n3 = (int(x) for x in fft_shape)
        h = C.c_void_p()
        check(LIB.addft_plan_create(C.byref(h), n1, n2, n3, int(m.shape[0]),
                                    m.ctypes.data_as(C.POINTER(C.c_int32))), "plan_create")
        self.handle = h
        self.shape = (n1, n2, n3)
        self.nG = int(m.shape[0])
        self.N = n1 * n2 * n3
        npl, ncol, ng = C.c_int(), C.c_int(), C.c_int()
        check(LIB.addft_plan_info(h, C.byref(npl), C.byref(ncol), C.byref(ng)), "plan_info")
        self.nplanes, self.ncols = npl.value, ncol.value

    def work_bytes(self, nbatch: int, dtype: int) -> int:
        return int(LIB.addft_work_bytes(self.handle, int(nbatch), int(dtype)))

    TUNING_KEYS = ("threads_plane", "threads_x", "xtile_kb", "slab_mb", "xline2", "plane2", "threads_plane2", "colfft",
                   "threads_xy", "xy_direct", "plane_split")

    def set_tuning(self, **kw) -> None:
        """Launch tunables of this plan (addft_plan_set_tuning)."""
        for k, v in kw.items():
            check(LIB.addft_plan_set_tuning(self.handle, k.encode(), int(v)), f"plan_set_tuning({k})")

    def get_tuning(self) -> dict:
        out = {}
        for k in self.TUNING_KEYS:
            v = C.c_long()
            check(LIB.addft_plan_get_tuning(self.handle, k.encode(), C.byref(v)), "plan_get_tuning")
            out[k] = int(v.value)
        return out

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                LIB.addft_plan_destroy(h)
            except Exception:
                pass
            self.handle = None


def _chunk_work(plan: Plan, dtype: int, nbatch: int, extra: int = 0, max_bytes: int = 1 << 30) -> torch.Tensor:
    per = plan.work_bytes(1, dtype) - (1 << 20)
    nfit = max(1, min(nbatch, (max_bytes - extra - (1 << 20)) // max(per, 1)))
    return workspace(extra + plan.work_bytes(nfit, dtype))


# ---------------------------------------------------------------------------
# transforms
# ---------------------------------------------------------------------------

def psi_to_real(plan: Plan, psi: torch.Tensor, omega: float) -> torch.Tensor:
    psi = _c(psi, "psi")
    lead = psi.shape[:-1]
    nb = int(np.prod(lead)) if lead else 1
    out = torch.empty(lead + (plan.N,), dtype=psi.dtype, device=psi.device)
    w = _chunk_work(plan, _dt(psi), nb)
    check(LIB.addft_psi_to_real(plan.handle, _dt(psi), nb, float(omega), _p(psi), _p(out), _p(w),
                                w.numel(), _stream()), "psi_to_real")
    return out


def real_to_psi(plan: Plan, psi_r: torch.Tensor, omega: float) -> torch.Tensor:
    psi_r = _c(psi_r, "psi_r")
    lead = psi_r.shape[:-1]
    nb = int(np.prod(lead)) if lead else 1
    out = torch.empty(lead + (plan.nG,), dtype=psi_r.dtype, device=psi_r.device)
    w = _chunk_work(plan, _dt(psi_r), nb)
    check(LIB.addft_real_to_psi(plan.handle, _dt(psi_r), nb, float(omega), _p(psi_r), _p(out), _p(w),
                                w.numel(), _stream()), "real_to_psi")
    return out


def kinetic(plan: Plan, bvec, kpts, dtype=torch.float64) -> torch.Tensor:
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
    out = torch.empty((kpts.shape[0], plan.nG), dtype=dtype, device="cuda")
    check(LIB.addft_kinetic(plan.handle, _dt(out), _d3(bvec), kpts.shape[0], _d3(kpts), _p(out), _stream()),
          "kinetic")
    return out


def projectors(plan: Plan, bvec, omega, kpts, pos, psp, dtype=torch.complex128) -> torch.Tensor:
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    P = pos.shape[0] * psp.nh
    out = torch.empty((kpts.shape[0], P, plan.nG), dtype=dtype, device="cuda")
    cs = psp.c_struct()
    check(LIB.addft_projectors(plan.handle, _dt(out), _d3(bvec), float(omega), kpts.shape[0], _d3(kpts),
                               pos.shape[0], _d3(pos), C.byref(cs), _p(out), _stream()), "projectors")
    return out


def hpsi_work_bytes(plan: Plan, dtype: int, nk: int, nb: int, nproj: int, chunk: int) -> int:
    return int(LIB.addft_hpsi_work_bytes(plan.handle, dtype, nk, nb, nproj, chunk))


def hpsi(plan: Plan, psi: torch.Tensor, kin: torch.Tensor, v_r: torch.Tensor, proj=None, dion=None,
         out=None, max_work: int = 1 << 30) -> torch.Tensor:
    """(T + V(r) + V_NL) psi for psi (nk, nb, nG) (ops/hpsi.py:35-50)."""
    psi = _c(psi, "psi")
    nk, nb, nG = psi.shape
    dt = _dt(psi)
    rdt = torch.float64 if dt == F64 else torch.float32
    kin = _c(kin.to(rdt), "kin")
    v_r = _c(v_r.to(rdt), "v_r")
    nproj = 0 if proj is None else int(proj.shape[1])
    if nproj:
        proj = _c(proj.to(psi.dtype), "proj")
        dion = _c(torch.as_tensor(dion, device=psi.device).to(rdt), "dion")
    if out is None:
        out = torch.empty_like(psi)
    per = plan.work_bytes(2, dt) - plan.work_bytes(1, dt)   # slab bytes per extra band in flight
    base = hpsi_work_bytes(plan, dt, nk, nb, nproj, 1)
    chunk = max(1, min(nk * nb, 1 + (max_work - base) // max(per, 1)))
    wb = hpsi_work_bytes(plan, dt, nk, nb, nproj, chunk)
    w = workspace(wb)
    check(LIB.addft_hpsi(plan.handle, dt, nk, nb, _p(psi), _p(kin), _p(v_r), nproj, _p(proj),
                         _p(dion), _p(out), _p(w), w.numel(), _stream()), "hpsi")
    return out


def hpsi_host(plan: Plan, psi_h: torch.Tensor, kin: torch.Tensor, v_r: torch.Tensor, proj=None, dion=None,
              out_h=None, chunk_bands: int = 32) -> torch.Tensor:
    """H psi of bands in (pinned) HOST memory (nk, nb, nG): the bands stream through the GPU in
    chunks with the upload, H psi and download of consecutive chunks overlapped (addft_hpsi_host).
    Returns the host result; the current stream is joined with the last download."""
    if psi_h.is_cuda:
        raise ValueError("psi_h must be a host tensor (pinned for overlapped copies)")
    psi_h = psi_h.contiguous()
    nk, nb, nG = psi_h.shape
    dt = _dt(psi_h)
    rdt = torch.float64 if dt == F64 else torch.float32
    kin = _c(kin.to(rdt), "kin")
    v_r = _c(v_r.to(rdt), "v_r")
    nproj = 0 if proj is None else int(proj.shape[1])
    if nproj:
        proj = _c(proj.to(psi_h.dtype), "proj")
        dion = _c(torch.as_tensor(dion, device=kin.device).to(rdt), "dion")
    if out_h is None:
        out_h = torch.empty_like(psi_h, pin_memory=psi_h.is_pinned())
    w = workspace(int(LIB.addft_hpsi_host_work_bytes(plan.handle, dt, nk, nb, nproj, int(chunk_bands))))
    check(LIB.addft_hpsi_host(plan.handle, dt, nk, nb, _p(psi_h), _p(kin), _p(v_r), nproj, _p(proj), _p(dion),
                              _p(out_h), int(chunk_bands), _p(w), w.numel(), _stream()), "hpsi_host")
    return out_h


def becp(proj: torch.Tensor, psi: torch.Tensor) -> torch.Tensor:
    proj, psi = _c(proj, "proj"), _c(psi, "psi")
    nk, nb, nG = psi.shape
    P = proj.shape[1]
    out = torch.empty((nk, P, nb), dtype=psi.dtype, device=psi.device)
    esz = 16 if _dt(psi) == F64 else 8
    w = workspace(max(256, 1300 * nk * P * nb * esz))
    check(LIB.addft_becp(_dt(psi), nk, nb, nG, P, _p(proj), _p(psi), _p(out), _p(w), w.numel(), _stream()),
          "becp")
    return out


def vnl_apply(proj, dion, becp_, hpsi_inout):
    nk, P, nb = becp_.shape
    nG = proj.shape[2]
    dt = _dt(hpsi_inout)
    rdt = torch.float64 if dt == F64 else torch.float32
    dion = _c(torch.as_tensor(dion, device="cuda").to(rdt), "dion")
    esz = 16 if dt == F64 else 8
    w = workspace(nk * P * nb * esz + 256)
    check(LIB.addft_vnl_apply(dt, nk, nb, nG, P, _p(_c(proj, "proj")), _p(dion), _p(_c(becp_, "becp")),
                              _p(hpsi_inout), _p(w), w.numel(), _stream()), "vnl_apply")
    return hpsi_inout


def nonlocal_energy(becp_, dion, wocc) -> torch.Tensor:
    nk, P, nb = becp_.shape
    dt = _dt(becp_)
    rdt = torch.float64 if dt == F64 else torch.float32
    dion = _c(torch.as_tensor(dion, device="cuda").to(rdt), "dion")
    wocc = _c(wocc.to(torch.float64), "wocc")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    esz = 16 if dt == F64 else 8
    w = workspace(nk * P * nb * esz + nk * nb * 8 + 1024)
    check(LIB.addft_nonlocal_energy(dt, nk, nb, P, _p(_c(becp_, "becp")), _p(dion), _p(wocc), _p(out), _p(w),
                                    w.numel(), _stream()), "nonlocal_energy")
    return out


def density(plan: Plan, psi: torch.Tensor, wocc: torch.Tensor, omega: float, out=None) -> torch.Tensor:
    """rho(r) = sum wocc |psi(r)|^2 (physics/density.py:18-23); wocc (nk, nb) = w_k f g_s."""
    psi = _c(psi, "psi")
    nk, nb, nG = psi.shape
    wocc = _c(wocc.to(torch.float64).reshape(-1), "wocc")
    if out is None:
        out = torch.empty(plan.N, dtype=torch.float64, device=psi.device)
    extra = ((8 * 8 * plan.N) + 255) // 256 * 256        # room for up to 8 per-split partial slabs
    w = _chunk_work(plan, _dt(psi), nk * nb, extra=extra)
    check(LIB.addft_density(plan.handle, _dt(psi), nk, nb, float(omega), _p(psi), _p(wocc), _p(out), _p(w),
                            w.numel(), _stream()), "density")
    return out


def xc_lda(rho: torch.Tensor, rho_dc=None, v_loc=None, v_h=None, want_vxc=True, want_veff=False):
    """PZ81: returns (v_xc or None, v_eff or None, sums[3] = {sum n eps_x, sum n eps_c, sum v_xc rho_dc})."""
    rho = _c(rho, "rho")
    n = rho.numel()
    v_xc = torch.empty_like(rho) if want_vxc else None
    v_eff = torch.empty_like(rho) if want_veff else None
    sums = torch.empty(3, dtype=torch.float64, device=rho.device)
    w = workspace(3 * 304 * 8 + 256)
    check(LIB.addft_xc_lda(n, _p(rho), _p(rho_dc), _p(v_loc), _p(v_h), _p(v_xc), _p(v_eff), _p(sums), _p(w),
                           w.numel(), _stream()), "xc_lda")
    return v_xc, v_eff, sums


def xc_lda_vjp(rho: torch.Tensor, g: torch.Tensor) -> torch.Tensor:
    rho, g = _c(rho, "rho"), _c(g.to(torch.float64), "g")
    out = torch.empty_like(rho)
    check(LIB.addft_xc_lda_vjp(rho.numel(), _p(rho), _p(g), _p(out), _stream()), "xc_lda_vjp")
    return out


def hartree(plan: Plan, bvec, omega, rho: torch.Tensor, want_potential=True):
    rho = _c(rho, "rho")
    v_h = torch.empty_like(rho) if want_potential else None
    e_h = torch.empty(1, dtype=torch.float64, device=rho.device)
    w = workspace(int(LIB.addft_hartree_work_bytes(plan.handle)))
    check(LIB.addft_hartree(plan.handle, _d3(bvec), float(omega), _p(rho), _p(v_h), _p(e_h), _p(w), w.numel(),
                            _stream()), "hartree")
    return v_h, e_h


def local_potential(rho_plan: Plan, bvec, omega, pos, psp) -> torch.Tensor:
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    out = torch.empty(rho_plan.N, dtype=torch.float64, device="cuda")
    w = workspace(int(LIB.addft_local_potential_work_bytes(rho_plan.handle)))
    cs = psp.c_struct()
    check(LIB.addft_local_potential(rho_plan.handle, _d3(bvec), float(omega), pos.shape[0], _d3(pos),
                                    C.byref(cs), _p(out), _p(w), w.numel(), _stream()), "local_potential")
    return out


def kerker(full_plan: Plan, bvec, x: torch.Tensor, alpha: float, gg0: float) -> torch.Tensor:
    """alpha * K x with the Kerker filter q^2/(q^2 + gg0) on the full box (scf.py:215-223)."""
    x = _c(x.to(torch.float64), "x")
    out = torch.empty_like(x)
    w = workspace(int(LIB.addft_kerker_work_bytes(full_plan.handle)))
    check(LIB.addft_kerker(full_plan.handle, _d3(bvec), _p(x), float(alpha), float(gg0), _p(out), _p(w), w.numel(),
                           _stream()), "kerker")
    return out


def zgemm_df(a: torch.Tensor, b: torch.Tensor, conj_a: bool = False, conj_b: bool = False,
             out: torch.Tensor = None) -> torch.Tensor:
    """op(a) @ op(b) for complex128 matrices (any strides; op = conjugate when asked) in
    double-float arithmetic on the FP32 pipes, ~1e-14 relative: the subspace products of
    the refinement (solver/davidson.py:48, :51-52, :59-61).  conj(x) @ y.T is
    zgemm_df(x, y.transpose(0, 1), conj_a=True) without a copy."""
    if a.dtype != torch.complex128 or b.dtype != torch.complex128 or not (a.is_cuda and b.is_cuda):
        raise TypeError("zgemm_df: complex128 CUDA tensors expected")
    M, K = a.shape
    K2, N = b.shape
    if K != K2:
        raise ValueError(f"zgemm_df: inner sizes {K} and {K2} differ")
    if out is None:
        out = torch.empty((M, N), dtype=torch.complex128, device=a.device)
    if out.shape != (M, N) or out.stride(1) != 1:
        raise ValueError("zgemm_df: out must be (M, N) with unit column stride")
    w = workspace(int(LIB.addft_zgemm_df_work_bytes(M, N, K)))
    check(LIB.addft_zgemm_df(M, N, K, _p(a), a.stride(0), a.stride(1), int(conj_a), _p(b), b.stride(0), b.stride(1),
                             int(conj_b), _p(out), out.stride(0), _p(w), w.numel(), _stream()), "zgemm_df")
    return out


def ewald(lattice, pos, charges, eta=0.9, nmax=8) -> torch.Tensor:
    """Device f64 [E, dE/dR (nat*3), dE/deps (9)] (physics/ewald.py:34-77)."""
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    nat = pos.shape[0]
    out = torch.empty(1 + 3 * nat + 9, dtype=torch.float64, device="cuda")
    w = workspace(int(LIB.addft_ewald_work_bytes(nat)))
    check(LIB.addft_ewald(_d3(lattice), nat, _d3(pos), _d3(charges), float(eta), int(nmax), _p(out), _p(w),
                          w.numel(), _stream()), "ewald")
    return out


def occupations(eig: torch.Tensor, kweights: torch.Tensor, nelec: float, sigma: float, gs: float = 2.0,
                iters: int = 80):
    """Fermi-Dirac occupations and mu on the device (occupation.py:25-49); integer filling for sigma < 1e-6."""
    eig = _c(eig.to(torch.float64), "eig")
    nk, nb = eig.shape
    kw = _c(kweights.to(torch.float64), "kweights")
    if sigma < 1e-6:
        return _integer_occupation(eig, kw, nelec, gs), torch.zeros(1, dtype=torch.float64, device="cuda")
    occ = torch.empty_like(eig)
    mu = torch.empty(1, dtype=torch.float64, device="cuda")
    check(LIB.addft_occupations(nk, nb, _p(eig), _p(kw), float(nelec), float(sigma), float(gs), int(iters),
                                _p(occ), _p(mu), _stream()), "occupations")
    return occ, mu


def _integer_occupation(eig, kw, nelec, gs):
    """T = 0 filling in ascending energy, last level fractional (occupation.py:52-65)."""
    neff = nelec / gs
    flat_e = eig.reshape(-1)
    flat_w = kw[:, None].expand(eig.shape).reshape(-1)
    order = torch.argsort(flat_e, stable=True)
    cum = torch.cumsum(flat_w[order], 0)
    filled = cum <= neff + 1e-12
    last = int(torch.argmax((cum > neff - 1e-12).to(torch.int32)))
    wl = flat_w[order][last]
    frac = torch.clamp((neff - (cum[last] - wl)) / wl, 0.0, 1.0)
    vals = torch.where(filled, 1.0, 0.0).to(torch.float64)
    if not bool(filled[last]):
        vals[last] = frac
    out = torch.zeros_like(flat_w)
    out[order] = vals
    return out.reshape(eig.shape)


def kinetic_stress(plan: Plan, bvec, kpts, psi, wocc) -> torch.Tensor:
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
    psi = _c(psi, "psi")
    nk, nb, _ = psi.shape
    out = torch.zeros(9, dtype=torch.float64, device="cuda")
    w = workspace(9 * 304 * 8 + 256)
    check(LIB.addft_kinetic_stress(plan.handle, _dt(psi), _d3(bvec), nk, _d3(kpts), nb, _p(psi),
                                   _p(_c(wocc.to(torch.float64), "wocc")), _p(out), _p(w), w.numel(), _stream()),
          "kinetic_stress")
    return out


def density_gradients(wfc_plan: Plan, rho_plan: Plan, bvec, omega, pos, psp, rho) -> torch.Tensor:
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    nat = pos.shape[0]
    out = torch.empty(5 + 3 * nat + 18, dtype=torch.float64, device="cuda")
    w = workspace(int(LIB.addft_density_gradients_work_bytes(wfc_plan.handle, rho_plan.handle, nat)))
    cs = psp.c_struct()
    check(LIB.addft_density_gradients(wfc_plan.handle, rho_plan.handle, _d3(bvec), float(omega), nat, _d3(pos),
                                      C.byref(cs), _p(_c(rho, "rho")), _p(out), _p(w), w.numel(), _stream()),
          "density_gradients")
    return out


def nonlocal_gradients(plan: Plan, bvec, omega, kpts, pos, psp, psi, wocc, dion) -> torch.Tensor:
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    psi = _c(psi, "psi")
    nk, nb, nG = psi.shape
    nat = pos.shape[0]
    dt = _dt(psi)
    rdt = torch.float64 if dt == F64 else torch.float32
    dion = _c(torch.as_tensor(dion, device="cuda").to(rdt), "dion")
    out = torch.empty(1 + 3 * nat + 9, dtype=torch.float64, device="cuda")
    w = workspace(int(LIB.addft_nonlocal_gradients_work_bytes(dt, nk, nb, nG, nat, psp.nh)))
    cs = psp.c_struct()
    check(LIB.addft_nonlocal_gradients(plan.handle, dt, _d3(bvec), float(omega), nk, _d3(kpts), nb, nat,
                                       _d3(pos), C.byref(cs), _p(psi), _p(_c(wocc.to(torch.float64), "wocc")),
                                       _p(dion), _p(out), _p(w), w.numel(), _stream()), "nonlocal_gradients")
    return out


# ---------------------------------------------------------------------------
# the reference's XLA FFI handlers (native/xc_lda.cu, native/pack.cu, native/eigh.cu),
# one C-ABI call each
# ---------------------------------------------------------------------------
def ffi_xc_lda(rho: torch.Tensor):
    """XcLdaHandler: (vxc, exc) with exc = sum n (eps_x + eps_c) at max(rho, 1e-14), a 0-d tensor."""
    rho = _c(rho.to(torch.float64), "rho")
    vxc = torch.empty_like(rho)
    exc = torch.empty((), dtype=torch.float64, device=rho.device)
    w = workspace(LIB.addft_ffi_xc_lda_work_bytes())
    check(LIB.addft_ffi_xc_lda(rho.numel(), _p(rho), _p(vxc), _p(exc), _p(w), w.numel(), _stream()), "ffi_xc_lda")
    return vxc, exc


def _idx32(idx: torch.Tensor) -> torch.Tensor:
    return _c(idx.to(device="cuda", dtype=torch.int32), "idx")


def ffi_scatter(coeffs: torch.Tensor, idx: torch.Tensor, nfft: int) -> torch.Tensor:
    """Scatter{C128,C64}Handler: out (batch, nfft) zero except out[b, idx[i]] = coeffs[b, i]."""
    coeffs = _c(coeffs, "coeffs")
    lead, nG = coeffs.shape[:-1], coeffs.shape[-1]
    batch = int(np.prod(lead)) if lead else 1
    idx = _idx32(idx)
    if idx.numel() != nG:
        raise ValueError("idx length != nG")
    out = torch.empty(lead + (int(nfft),), dtype=coeffs.dtype, device=coeffs.device)
    check(LIB.addft_ffi_scatter(_dt(coeffs), batch, nG, int(nfft), _p(coeffs), _p(idx), _p(out), _stream()),
          "ffi_scatter")
    return out


def ffi_gather(grid: torch.Tensor, idx: torch.Tensor, nG: int) -> torch.Tensor:
    """Gather{C128,C64}Handler: out[b, i] = grid[b, idx[i]]."""
    grid = _c(grid, "grid")
    lead, nfft = grid.shape[:-1], grid.shape[-1]
    batch = int(np.prod(lead)) if lead else 1
    idx = _idx32(idx)
    if idx.numel() != int(nG):
        raise ValueError("idx length != nG")
    out = torch.empty(lead + (int(nG),), dtype=grid.dtype, device=grid.device)
    check(LIB.addft_ffi_gather(_dt(grid), batch, int(nG), nfft, _p(grid), _p(idx), _p(out), _stream()),
          "ffi_gather")
    return out


def ffi_index_in_range(idx: torch.Tensor, nfft: int) -> bool:
    """True if every index lies in [0, nfft) (synchronises)."""
    idx = _idx32(idx)
    bad = torch.empty(1, dtype=torch.int32, device=idx.device)
    check(LIB.addft_ffi_check_index(idx.numel(), int(nfft), _p(idx), _p(bad), _stream()), "ffi_check_index")
    return int(bad.item()) == 0


def ffi_eigh_lowest(H: torch.Tensor, nband: int):
    """EighLowestHandler: H (nk, n, n) complex128 Hermitian -> eig (nk, nband), vec (nk, nband, n)."""
    H = _c(H.to(torch.complex128), "H")
    nk, n = H.shape[0], H.shape[1]
    if H.shape != (nk, n, n):
        raise ValueError("H must be (nk, n, n)")
    eig = torch.empty((nk, int(nband)), dtype=torch.float64, device=H.device)
    vec = torch.empty((nk, int(nband), n), dtype=torch.complex128, device=H.device)
    nbytes = LIB.addft_ffi_eigh_lowest_work_bytes(nk, n)
    if nbytes == 0:
        raise _lib.AddftError("ffi_eigh_lowest: cuSOLVER is not available: " +
                              LIB.addft_last_error().decode(errors="replace"))
    w = workspace(nbytes)
    check(LIB.addft_ffi_eigh_lowest(nk, n, int(nband), _p(H), _p(eig), _p(vec), _p(w), w.numel(), _stream()),
          "ffi_eigh_lowest")
    return eig, vec
