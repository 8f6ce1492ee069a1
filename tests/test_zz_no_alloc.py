"""addft_hpsi_noalloc: H psi for callers that may not allocate device memory.

Such callers (an XLA FFI handler inside a JAX program, where the framework
has pre-reserved most of the device memory; an application under a fixed
device-memory budget) cannot hand the library a freshly allocated work
buffer, so this entry point takes its scratch from a static array inside the
library.  The test calls it through the C ABI and checks it against
addft_hpsi (which uses a caller work buffer) on the same inputs, twice in a
row, since every call reuses the same static scratch.  Tolerance: the FP64
parity bar of the other H psi tests (1e-10), FP32 at 1e-6 relative.

This file is named so pytest collects it last.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import FRAC_DISTORTED, LATTICE, gpu_available

pytestmark = pytest.mark.gpu
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import torch  # noqa: E402

import addft_gb300 as ad  # noqa: E402
from addft_gb300 import ops  # noqa: E402
from addft_gb300._lib import LIB  # noqa: E402
from addft_gb300.system import build_geometry_cache  # noqa: E402


def _p(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _noalloc(plan, dt, psi, kin, v, proj, dion, out):
    nk, nb, _ = psi.shape
    nproj = 0 if proj is None else proj.shape[1]
    return LIB.addft_hpsi_noalloc(plan.handle, dt, nk, nb, _p(psi), _p(kin), _p(v), nproj, _p(proj), _p(dion),
                                  _p(out), _stream())


def _inputs(dtype, kmesh=None, nband=3):
    s = ad.setup(LATTICE, FRAC_DISTORTED, ecut=2.0, nband=nband, density_factor=4.0,
                 kmesh=ad.monkhorst_pack(kmesh) if kmesh else None)
    cache = build_geometry_cache(s.geo, s.static)
    rng = np.random.default_rng(17)
    nk, nG = s.static.nk, s.static.basis.nG
    psi = torch.as_tensor(rng.normal(size=(nk, nband, nG)) + 1j * rng.normal(size=(nk, nband, nG)), device="cuda")
    v = torch.as_tensor(rng.uniform(-1, 1, s.static.basis.nfft), device="cuda")
    if dtype == "fp64":
        return s, psi, cache.kin, v, cache.proj, cache.dion
    p32, d32, k32 = cache.f32()
    return s, psi.to(torch.complex64), k32, v.to(torch.float32), p32, d32


@pytest.mark.parametrize("prec,kmesh", [("fp64", None), ("fp64", (2, 2, 2)), ("fp32", None)])
def test_noalloc_matches_hpsi_on_two_calls(prec, kmesh):
    s, psi, kin, v, proj, dion = _inputs(prec, kmesh)
    plan = s.static.device().wfc
    ref = ops.hpsi(plan, psi, kin, v, proj, dion)
    dt = 1 if prec == "fp64" else 0
    tol = 1e-10 if prec == "fp64" else 1e-6
    for _ in range(2):
        out = torch.full_like(psi, float("nan"))
        assert _noalloc(plan, dt, psi, kin, v, proj, dion, out) == 0, LIB.addft_last_error()
        torch.cuda.synchronize()
        err = float((out - ref).abs().max() / ref.abs().max())
        assert err < tol


def test_noalloc_chunks_a_large_box_and_rejects_oversize():
    # 72^3 box, 8 FP32 bands: the 8 MiB scratch holds about two band slabs,
    # so the call runs several band chunks back to back.
    n = 72
    r = int(0.45 * n)
    m = np.stack(np.meshgrid(*(np.arange(-r, r + 1),) * 3, indexing="ij"), -1).reshape(-1, 3)
    m = m[np.sum(m * m, axis=1) <= (0.45 * n) ** 2].astype(np.int32)
    plan = ops.Plan((n, n, n), m)
    rng = np.random.default_rng(3)
    psi = torch.as_tensor(rng.normal(size=(1, 8, len(m))) + 1j * rng.normal(size=(1, 8, len(m))),
                          device="cuda").to(torch.complex64)
    kin = torch.as_tensor(rng.uniform(0, 5, (1, len(m))), device="cuda").to(torch.float32)
    v = torch.as_tensor(rng.uniform(-1, 1, n ** 3), device="cuda").to(torch.float32)
    ref = ops.hpsi(plan, psi, kin, v)
    for _ in range(2):
        out = torch.zeros_like(psi)
        assert _noalloc(plan, 0, psi, kin, v, None, None, out) == 0, LIB.addft_last_error()
        torch.cuda.synchronize()
        assert float((out - ref).abs().max() / ref.abs().max()) < 1e-6
    # FP64 slab of this box (~5.5 MB) plus buffers still fits; a 96^3 FP64 sphere does not
    n2 = 96
    r2 = int(0.45 * n2)
    m2 = np.stack(np.meshgrid(*(np.arange(-r2, r2 + 1),) * 3, indexing="ij"), -1).reshape(-1, 3)
    m2 = m2[np.sum(m2 * m2, axis=1) <= (0.45 * n2) ** 2].astype(np.int32)
    big = ops.Plan((n2, n2, n2), m2)
    need = LIB.addft_hpsi_work_bytes(big.handle, 1, 1, 1, 0, 1)
    assert need > LIB.addft_hpsi_noalloc_max_scratch_bytes()
    psi2 = torch.zeros((1, 1, len(m2)), dtype=torch.complex128, device="cuda")
    out2 = torch.zeros_like(psi2)
    kin2 = torch.zeros((1, len(m2)), dtype=torch.float64, device="cuda")
    v2 = torch.zeros(n2 ** 3, dtype=torch.float64, device="cuda")
    st = _noalloc(big, 1, psi2, kin2, v2, None, None, out2)
    assert st == 5 and b"static scratch" in LIB.addft_last_error()


def _sphere_plan(n):
    r = int(0.45 * n)
    m = np.stack(np.meshgrid(*(np.arange(-r, r + 1),) * 3, indexing="ij"), -1).reshape(-1, 3)
    m = m[np.sum(m * m, axis=1) <= (0.45 * n) ** 2].astype(np.int32)
    return ops.Plan((n, n, n), m), len(m)


def test_noalloc_projector_heavy_case_runs_without_split_partials():
    """8 k points x 64 bands x 32 projectors in FP64: the split-K partials of becp at the
    default number of splits alone exceed the static scratch, but the minimum (becp arrays
    plus one band of FFT scratch) fits, so the call runs with fewer splits."""
    plan, nG = _sphere_plan(24)
    nk, nb, P = 8, 64, 32
    need_default = LIB.addft_hpsi_work_bytes(plan.handle, 1, nk, nb, P, 1)
    assert need_default > LIB.addft_hpsi_noalloc_max_scratch_bytes()
    g = torch.Generator(device="cuda").manual_seed(11)
    psi = torch.randn((nk, nb, nG), dtype=torch.complex128, device="cuda", generator=g)
    proj = torch.randn((nk, P, nG), dtype=torch.complex128, device="cuda", generator=g)
    kin = torch.rand((nk, nG), dtype=torch.float64, device="cuda", generator=g)
    v = torch.rand(24 ** 3, dtype=torch.float64, device="cuda", generator=g) - 0.5
    d = torch.randn((P, P), dtype=torch.float64, device="cuda", generator=g)
    dion = 0.5 * (d + d.T)
    ref = ops.hpsi(plan, psi, kin, v, proj, dion)
    for _ in range(2):
        out = torch.full_like(psi, float("nan"))
        assert _noalloc(plan, 1, psi, kin, v, proj, dion, out) == 0, LIB.addft_last_error()
        torch.cuda.synchronize()
        assert float((out - ref).abs().max() / ref.abs().max()) < 1e-10


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """After the first call on the device (which resolves the scratch array's address and
    loads the kernels), a call that runs several band chunks frees and allocates nothing:
    the device's free memory is the same before and after it."""
    plan, nG = _sphere_plan(72)
    g = torch.Generator(device="cuda").manual_seed(5)
    psi = torch.randn((1, 8, nG), dtype=torch.complex64, device="cuda", generator=g)
    kin = torch.rand((1, nG), dtype=torch.float32, device="cuda", generator=g)
    v = torch.rand(72 ** 3, dtype=torch.float32, device="cuda", generator=g)
    out = torch.empty_like(psi)
    assert _noalloc(plan, 0, psi, kin, v, None, None, out) == 0, LIB.addft_last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert _noalloc(plan, 0, psi, kin, v, None, None, out) == 0, LIB.addft_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free0 == free1
