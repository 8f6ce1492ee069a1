"""Per-plan launch tuning, the graph-captured batch of structures, the autotuner.

Graph replay must reproduce the eager launch sequence bit for bit; any tuning
must keep FP32 H psi within the FP32 tolerance of the FP64 kernels (2e-3 is
the reference's FP32 H psi bar, test_hpsi.py:53-72; these land near 1e-6).
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import torch  # noqa: E402

from addft_gb300 import ops  # noqa: E402
from addft_gb300._lib import AddftError  # noqa: E402
from addft_gb300.batch import HpsiBatch, items_from_systems, silicon_batch  # noqa: E402


@pytest.fixture(scope="module")
def small_batch():
    systems = silicon_batch(ecut=4.0, kmesh=(2, 2, 2))[:4]       # Si2, Si4, Si8 x2
    return systems, items_from_systems(systems)


def _fp64(it):
    return ops.hpsi(it.plan, it.psi.to(torch.complex128), it.kin.double(), it.v.double(),
                    it.proj.to(torch.complex128), it.dion.double())


def test_plan_tuning_round_trip_and_validation(small_batch):
    plan = small_batch[1][0].plan
    old = plan.get_tuning()
    plan.set_tuning(plane2=0, xline2=0, threads_plane=128, slab_mb=32)
    t = plan.get_tuning()
    assert (t["plane2"], t["xline2"], t["threads_plane"], t["slab_mb"]) == (0, 0, 128, 32)
    with pytest.raises(AddftError):
        plan.set_tuning(threads_plane=100)
    with pytest.raises(AddftError):
        plan.set_tuning(no_such_key=1)
    plan.set_tuning(**old)
    assert plan.get_tuning() == old


def test_graph_replay_matches_eager_and_fp64(small_batch):
    _, items = small_batch
    b = HpsiBatch(items)
    b.run_eager()
    torch.cuda.synchronize()
    eager = [it.out.clone() for it in items]
    for branches in (1, 3):
        for it in items:
            it.out.zero_()
        b.capture(branches=branches)
        b.run()
        torch.cuda.synchronize()
        for it, e in zip(items, eager):
            assert torch.equal(it.out, e)
        ref = _fp64(it)
        assert float((it.out.to(torch.complex128) - ref).abs().max() / ref.abs().max()) < 1e-5


def test_autotuner_picks_a_candidate_and_keeps_results(small_batch):
    _, items = small_batch
    cands = [{"plane2": 1, "xline2": 1, "slab_mb": 96, "threads_plane": 256},
             {"plane2": 0, "xline2": 1, "slab_mb": 32, "threads_plane": 128},
             {"plane2": 0, "xline2": 0, "slab_mb": 256, "threads_plane": 256}]
    b = HpsiBatch(items)
    chosen = b.tune(candidates=cands, reps=2)
    assert len(chosen) == len(items)
    for it, ch in zip(items, chosen):
        t = it.plan.get_tuning()
        assert {k: t[k] for k in ("plane2", "xline2", "slab_mb", "threads_plane")} in cands
        assert ch["ms"] > 0
    b.run()
    torch.cuda.synchronize()
    for it in items:
        ref = _fp64(it)
        assert float((it.out.to(torch.complex128) - ref).abs().max() / ref.abs().max()) < 1e-5


def test_graph_replay_structure_matches_oracle(small_batch):
    """One structure of the captured batch (Si4, tetragonal cell, 2x2x2 k mesh) against the
    NumPy oracle's H psi per k point (pw.hpsi_tables), with the oracle's own projector,
    kinetic and D tables of the same cell: FP32 within 1e-5 of max |H psi|."""
    from oracle import pw
    systems, items = small_batch
    b = HpsiBatch(items)
    b.capture(branches=2)
    b.run()
    torch.cuda.synchronize()
    s, it = systems[1], items[1]
    o = pw.setup(s.geo.lattice, s.geo.frac, ecut=4.0, nband=s.static.nband, kmesh=pw.monkhorst_pack((2, 2, 2)))
    assert np.array_equal(o.static.basis.miller, s.static.basis.miller)
    proj = pw.projectors(o.static, o.lattice, o.frac)
    dion = pw.dion_full(o.static.psp, o.static.natom)
    v = it.v.double().cpu().numpy()
    psi = it.psi.to(torch.complex128).cpu().numpy()
    out = it.out.to(torch.complex128).cpu().numpy()
    for ik, kp in enumerate(o.static.kpts):
        kin = pw.kinetic_diag(o.static.basis, o.lattice, kp)
        ref = pw.hpsi_tables(o.static.basis.fft_shape, o.static.basis.miller, psi[ik], kin, v, proj[ik], dion)
        assert np.max(np.abs(out[ik] - ref)) / np.max(np.abs(ref)) < 1e-5, ik
