"""Oracle parity of H psi on the microbench's large boxes (48^3, 72^3, 75^3).

The benchmarked step is one FP32 H psi on the 72^3 microbench sphere with
8 atoms x 4 projectors.  These tests run exactly that workload generator
(``bench.host_workload`` / ``bench.host_tables``: seeded orthonormal bands,
V_loc of 16 plane waves, projectors from the reference formulas) through the
C ABI and compare with the NumPy oracle's H psi (``pw.hpsi_tables``, the
restatement of ops/hpsi.py:35-50), not with the library's own FP64 kernels.
The FP32 runs take the kernels the bench times: the column pipeline (z-column
inverse, xy-plane kernel with V(r) between the two transforms, z-column forward
with the kinetic term), the mma.sync becp on its forked stream and the tcgen05
V_NL apply.

Tolerances (relative to max |H psi|): FP64 1e-10 (the reference's H psi bar,
tests/test_hpsi.py:15-32), FP32 1e-5 (the FP32 H psi lands near 2e-6; the
reference's own FP32 bar is 2e-3, tests/test_hpsi.py:53-72).
"""

from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import torch  # noqa: E402

import bench  # noqa: E402
from addft_gb300 import ops  # noqa: E402
from addft_gb300.geometry import reciprocal, volume  # noqa: E402
from addft_gb300.psp import Pseudo  # noqa: E402
from oracle import pw  # noqa: E402

TOL = {"fp64": 1e-10, "fp32": 1e-5}
WORKERS = os.cpu_count()


def _device_tables(wl, plan, cdt, rdt):
    """Kinetic, projector and D tables built by the library (as bench.py does)."""
    lat = wl["lat"]
    psp = Pseudo(proj_w=(1.0, 1.0), proj_b=(1.0, 1.0), proj_l=(0, 1), dion=np.eye(2))
    kin = ops.kinetic(plan, reciprocal(lat), np.zeros((1, 3)), dtype=rdt)
    proj = ops.projectors(plan, reciprocal(lat), volume(lat), np.zeros((1, 3)), wl["pos"], psp, dtype=cdt)
    P = proj.shape[1]
    return kin, proj, torch.eye(P, dtype=rdt, device="cuda")


@pytest.fixture(scope="module", params=[48, 72, 75])
def box_case(request):
    n = request.param
    wl = bench.host_workload(n=n, nb=3)
    kin, proj, dion = bench.host_tables(wl)
    ref = pw.hpsi_tables((n,) * 3, wl["miller"], wl["psi"], kin, wl["v"], proj, dion, workers=WORKERS)
    return wl, (kin, proj, dion), ref


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_hpsi_microbench_box_matches_oracle(box_case, prec):
    wl, (okin, oproj, _), ref = box_case
    n, nb, nG = wl["n"], wl["nb"], wl["nG"]
    cdt, rdt = (torch.complex128, torch.float64) if prec == "fp64" else (torch.complex64, torch.float32)
    plan = ops.Plan((n,) * 3, wl["miller"])
    kin, proj, dion = _device_tables(wl, plan, cdt, rdt)
    # the library's tables agree with the oracle's before H psi uses them
    ptol = 1e-13 if prec == "fp64" else 1e-6
    assert np.max(np.abs(proj[0].cpu().numpy() - oproj)) / np.max(np.abs(oproj)) < ptol
    assert np.max(np.abs(kin[0].cpu().numpy() - okin)) / np.max(okin) < ptol
    psi = torch.as_tensor(wl["psi"], device="cuda").to(cdt).reshape(1, nb, nG).contiguous()
    v = torch.as_tensor(wl["v"], device="cuda").to(rdt)
    out = ops.hpsi(plan, psi, kin, v, proj, dion)[0].cpu().numpy()
    err = np.max(np.abs(out - ref)) / np.max(np.abs(ref))
    assert err < TOL[prec], (n, prec, err)


def test_hpsi_benchmark_workload_all_64_bands_fp32():
    """The full benchmarked step (72^3, 64 bands, 8 atoms x 4 projectors, FP32) against the oracle:
    same launch shapes as the timed step (one 64-band becp tile, all bands in flight)."""
    wl = bench.host_workload()
    kin_o, proj_o, dion_o = bench.host_tables(wl)
    n, nb, nG = wl["n"], wl["nb"], wl["nG"]
    ref = pw.hpsi_tables((n,) * 3, wl["miller"], wl["psi"], kin_o, wl["v"], proj_o, dion_o, workers=WORKERS)
    plan = ops.Plan((n,) * 3, wl["miller"])
    kin, proj, dion = _device_tables(wl, plan, torch.complex64, torch.float32)
    psi = torch.as_tensor(wl["psi"], device="cuda").to(torch.complex64).reshape(1, nb, nG).contiguous()
    v = torch.as_tensor(wl["v"], device="cuda").to(torch.float32)
    out = ops.hpsi(plan, psi, kin, v, proj, dion)[0].cpu().numpy()
    err_band = np.max(np.abs(out - ref), axis=1) / np.max(np.abs(ref), axis=1)
    assert np.all(err_band < TOL["fp32"]), err_band.max()
    # size-independent checks at full size: H is Hermitian and its Rayleigh quotients are real
    psi64 = wl["psi"]
    hmat = psi64.conj() @ out.T
    assert np.max(np.abs(hmat - hmat.conj().T)) / np.max(np.abs(hmat)) < 1e-5


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_hpsi_is_linear_on_the_largest_box(prec):
    """Size-independent check at the largest microbench box (75^3, 64 bands, 8 atoms x 4
    projectors): H (a psi1 + b psi2) = a H psi1 + b H psi2 for complex a, b, all three band sets in
    one call (96 bands: the band-tiled becp, the apply and the FFT batching see mixed inputs).
    FP64 within 1e-12 and FP32 within 3e-5 of max |H psi| (three FP32 results of ~2e-6 error each,
    two of them scaled by |a| = 1 and |b| = 1.32)."""
    wl = bench.host_workload(n=75)
    n, nb, nG = wl["n"], wl["nb"], wl["nG"]
    cdt, rdt = (torch.complex128, torch.float64) if prec == "fp64" else (torch.complex64, torch.float32)
    plan = ops.Plan((n,) * 3, wl["miller"])
    kin, proj, dion = _device_tables(wl, plan, cdt, rdt)
    h = nb // 2
    p1, p2 = wl["psi"][:h], wl["psi"][h:2 * h]
    a, b = 0.6 - 0.8j, -1.3 + 0.25j
    psi = np.concatenate([p1, p2, a * p1 + b * p2])
    psi = torch.as_tensor(psi, device="cuda").to(cdt).reshape(1, 3 * h, nG).contiguous()
    v = torch.as_tensor(wl["v"], device="cuda").to(rdt)
    out = ops.hpsi(plan, psi, kin, v, proj, dion)[0].cpu().numpy().astype(np.complex128)
    lhs, rhs = out[2 * h:], a * out[:h] + b * out[h:2 * h]
    err = np.max(np.abs(lhs - rhs)) / np.max(np.abs(out))
    assert err < (1e-12 if prec == "fp64" else 3e-5), (prec, err)


@pytest.mark.parametrize("slab_mb", [200, 4])
def test_hpsi_persistent_pipeline_matches_oracle(box_case, slab_mb):
    """The column pipeline as one persistent kernel (tuning colfft = 2: CTAs take z-column and
    xy-plane work items band by band, with dependency counters) on the same workload, two k points
    of the same bands, all bands in one launch (slab_mb 200) or one band per launch (4, so the
    launches start at band offsets > 0): FP32 within 1e-5 of the oracle, no expired wait."""
    from addft_gb300._lib import LIB
    wl, (okin, oproj, _), ref = box_case
    n, nb, nG = wl["n"], wl["nb"], wl["nG"]
    plan = ops.Plan((n,) * 3, wl["miller"])
    plan.set_tuning(colfft=2, slab_mb=slab_mb)
    kin, proj, dion = _device_tables(wl, plan, torch.complex64, torch.float32)
    psi1 = torch.as_tensor(wl["psi"], device="cuda").to(torch.complex64).reshape(1, nb, nG)
    psi = torch.cat([psi1, psi1.flip(1)], 0).contiguous()          # k = 0, 1 (same k vector)
    kin2, proj2 = kin.repeat(2, 1).contiguous(), proj.repeat(2, 1, 1).contiguous()
    v = torch.as_tensor(wl["v"], device="cuda").to(torch.float32)
    LIB.addft_hpsi_fused_status()
    out = ops.hpsi(plan, psi, kin2, v, proj2, dion).cpu().numpy()
    assert LIB.addft_hpsi_fused_status() == 0
    for k, r in ((0, ref), (1, ref[::-1])):
        err = np.max(np.abs(out[k] - r)) / np.max(np.abs(r))
        assert err < TOL["fp32"], (n, slab_mb, k, err)


@pytest.mark.parametrize("prec,chunk", [("fp32", 24), ("fp32", 8), ("fp64", 24)])
def test_hpsi_host_buffers_match_device_call(prec, chunk):
    """addft_hpsi_host (bands in pinned host memory, streamed through the GPU in chunks with
    the copies overlapped) equals addft_hpsi on the same bands: two k points, chunks that do
    not divide the band count.  FP32 within 1e-6 and FP64 within 1e-12 of max |H psi| (only
    the becp split-sum order differs)."""
    wl = bench.host_workload(n=48, nb=40)
    n, nb, nG = wl["n"], wl["nb"], wl["nG"]
    cdt, rdt = (torch.complex128, torch.float64) if prec == "fp64" else (torch.complex64, torch.float32)
    plan = ops.Plan((n,) * 3, wl["miller"])
    kin, proj, dion = _device_tables(wl, plan, cdt, rdt)
    psi1 = torch.as_tensor(wl["psi"]).to(cdt).reshape(1, nb, nG)
    psi_h = torch.cat([psi1, psi1.flip(1)], 0).contiguous().pin_memory()
    kin2, proj2 = kin.repeat(2, 1).contiguous(), proj.repeat(2, 1, 1).contiguous()
    v = torch.as_tensor(wl["v"], device="cuda").to(rdt)
    ref = ops.hpsi(plan, psi_h.cuda(), kin2, v, proj2, dion).cpu()
    out = ops.hpsi_host(plan, psi_h, kin2, v, proj2, dion, chunk_bands=chunk)
    torch.cuda.current_stream().synchronize()
    err = float((out - ref).abs().max() / ref.abs().max())
    assert err < (1e-12 if prec == "fp64" else 1e-6), err


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("n", [15, 48, 72])
def test_hpsi_and_density_match_reference_code(n, prec):
    """H psi and the band density on the microbench workload against the values the reference's
    own ops/hpsi.py and physics/density.py produced (tests/golden/make_reference_fixtures.py):
    1e-10 relative in FP64, 1e-5 in FP32 (the kernels the bench times)."""
    from test_reference_fixtures import FIX, assert_micro
    m = FIX["microbench"][str(n)]
    wl = bench.host_workload(n=n, nb=m["nb"])
    nb, nG = wl["nb"], wl["nG"]
    cdt, rdt = (torch.complex128, torch.float64) if prec == "fp64" else (torch.complex64, torch.float32)
    plan = ops.Plan((n,) * 3, wl["miller"])
    kin, proj, dion = _device_tables(wl, plan, cdt, rdt)
    psi = torch.as_tensor(wl["psi"], device="cuda").to(cdt).reshape(1, nb, nG).contiguous()
    v = torch.as_tensor(wl["v"], device="cuda").to(rdt)
    h = ops.hpsi(plan, psi, kin, v, proj, dion)[0].cpu().numpy().astype(np.complex128)
    w = torch.full((1, nb), 2.0, dtype=torch.float64, device="cuda")
    rho = ops.density(plan, psi, w, volume(wl["lat"])).cpu().numpy()
    assert_micro(h, rho, m, 1e-10 if prec == "fp64" else 1e-5)
