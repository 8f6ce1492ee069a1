"""Batched H psi of several structures in one captured CUDA graph, with an
autotuner for the per-box launch shapes.

A batch holds, for every structure, the FP32 tables of its H psi (plan of its
wavefunction shell and FFT box, kinetic diagonal, V(r), projectors, D) and
device-resident psi / output / scratch buffers that it owns, so the pointers a
captured graph records stay valid.  ``tune`` picks, per structure, the plan
tunables (two-pass register kernels on or off, generic-kernel CTA sizes and
the slab bytes per band chunk, i.e. how many bands one launch sequence
carries) by timing candidates with CUDA events; ``capture`` records all
structures' H psi -- every band and k point -- as one graph, and ``run``
replays it.  There is no counterpart in the reference, whose JAX path runs
one structure per jit call.
"""

from __future__ import annotations

import ctypes as C
import itertools
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import ops
from ._lib import LIB, check

F32 = 0


@dataclass
class BatchItem:
    plan: ops.Plan
    psi: torch.Tensor        # (nk, nb, nG) complex64
    kin: torch.Tensor        # (nk, nG) float32
    v: torch.Tensor          # (N,) float32
    proj: torch.Tensor       # (nk, P, nG) complex64
    dion: torch.Tensor       # (P, P) float32
    out: torch.Tensor = None
    work: torch.Tensor = None
    tuning: dict = field(default_factory=dict)

    @property
    def bands(self) -> int:
        return int(self.psi.shape[0] * self.psi.shape[1])


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class HpsiBatch:
    """H psi over all bands and k points of several structures (FP32)."""

    def __init__(self, items, max_work: int = 1 << 30):
        self.items = list(items)
        self.max_work = int(max_work)
        self.graph = None
        for it in self.items:
            it.out = torch.empty_like(it.psi)
            self._size_work(it)

    def _size_work(self, it: BatchItem) -> None:
        nk, nb, _ = it.psi.shape
        P = int(it.proj.shape[1])
        need = int(LIB.addft_hpsi_work_bytes(it.plan.handle, F32, nk, nb, P, nk * nb))
        floor = int(LIB.addft_hpsi_work_bytes(it.plan.handle, F32, nk, nb, P, 1))
        nbytes = max(floor, min(need, self.max_work))
        if it.work is None or it.work.numel() < nbytes:
            it.work = torch.empty(nbytes + 256, dtype=torch.uint8, device="cuda")
        self.graph = None

    def _launch(self, it: BatchItem) -> None:
        nk, nb, _ = it.psi.shape
        P = int(it.proj.shape[1])
        base = (it.work.data_ptr() + 255) & ~255
        check(LIB.addft_hpsi(it.plan.handle, F32, nk, nb, _p(it.psi), _p(it.kin), _p(it.v), P, _p(it.proj),
                             _p(it.dion), _p(it.out), C.c_void_p(base), it.work.numel() - (base - it.work.data_ptr()),
                             _stream()), "hpsi (batch)")

    def run_eager(self) -> None:
        for it in self.items:
            self._launch(it)

    def capture(self, branches: int = 4) -> None:
        """Record every structure's H psi as one CUDA graph (after a warm-up launch).
        With ``branches`` > 1 the structures are dealt, largest first, onto that many
        streams forked from and joined to the capture stream, so the graph has
        parallel branches and small boxes overlap large ones."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run_eager()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        order = sorted(self.items, key=lambda it: -it.bands * it.plan.N)
        nbr = max(1, min(int(branches), len(order)))
        lanes = [[] for _ in range(nbr)]
        load = [0.0] * nbr
        for it in order:                               # greedy: least-loaded branch
            j = int(np.argmin(load))
            lanes[j].append(it)
            load[j] += it.bands * it.plan.N * np.log2(it.plan.N)
        self.branch_streams = [torch.cuda.Stream() for _ in range(nbr)]
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            main = torch.cuda.current_stream()
            fork = torch.cuda.Event()
            fork.record(main)
            joins = []
            for st, lane in zip(self.branch_streams, lanes):
                st.wait_event(fork)
                with torch.cuda.stream(st):
                    for it in lane:
                        self._launch(it)
                e = torch.cuda.Event()
                e.record(st)
                joins.append(e)
            for e in joins:
                main.wait_event(e)
        torch.cuda.synchronize()
        self.graph = g

    def run(self) -> None:
        if self.graph is None:
            self.capture()
        self.graph.replay()

    @property
    def bands(self) -> int:
        return sum(it.bands for it in self.items)

    # -- autotuning ----------------------------------------------------------
    def tune(self, candidates=None, reps: int = 3, verbose: bool = False) -> list:
        """Per structure, time each candidate tuning (CUDA events, best of ``reps``)
        and keep the fastest; returns the chosen tunings."""
        cands = candidates or default_candidates()
        chosen = []
        for it in self.items:
            best, best_t = None, float("inf")
            for cand in cands:
                it.plan.set_tuning(**cand)
                self._size_work(it)
                self._launch(it)                       # warm / shared-memory opt-in
                t = _time_cuda(lambda: self._launch(it), reps)
                if verbose:
                    print(it.plan.shape, cand, f"{1e3 * t:.3f} ms")
                if t < best_t:
                    best, best_t = dict(cand), t
            it.plan.set_tuning(**best)
            it.tuning = dict(best, ms=1e3 * best_t)
            self._size_work(it)
            chosen.append(it.tuning)
        self.graph = None
        return chosen


def default_candidates() -> list:
    """Column pipeline (xy-plane CTA sizes) or plane pipeline (two-pass kernels on/off x
    generic CTA sizes) x slab bytes per band chunk."""
    out = []
    for slab in (32, 96, 256):
        for txy in (128, 256, 384):
            out.append({"colfft": 1, "threads_xy": txy, "slab_mb": slab})
    for plane2, xline2, slab in itertools.product((1, 0), (1, 0), (32, 96, 256)):
        for tp in ((256,) if plane2 else (128, 256)):
            out.append({"colfft": 0, "plane2": plane2, "xline2": xline2, "slab_mb": slab, "threads_plane": tp})
    return out


def _time_cuda(fn, reps: int) -> float:
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b) / 1e3)
    return best


def items_from_systems(systems, seed: int = 7) -> list:
    """FP32 H psi inputs for each System: orthonormal random bands (seeded), V(r) =
    the effective potential of the uniform initial density, the geometry's
    projectors and D."""
    from .solver import effective_potential, initial_density
    from .system import build_geometry_cache
    items = []
    g = torch.Generator(device="cuda").manual_seed(seed)
    for s in systems:
        st = s.static
        cache = build_geometry_cache(s.geo, st)
        v, _ = effective_potential(st, cache, initial_density(st, cache))
        nk, nb, nG = st.nk, st.nband, st.basis.nG
        psi = torch.randn((nk, nb, nG), dtype=torch.complex128, device="cuda", generator=g)
        for k in range(nk):
            q, _ = torch.linalg.qr(psi[k].transpose(0, 1))
            psi[k] = q.transpose(0, 1)
        proj32, dion32, kin32 = cache.f32()
        items.append(BatchItem(plan=st.device().wfc, psi=psi.to(torch.complex64).contiguous(), kin=kin32,
                               v=v.to(torch.float32).contiguous(), proj=proj32, dion=dion32))
    return items


def timed(fn, steps: int, warmup: int = 3):
    """Seconds per call of fn with CUDA events, after warm-up."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3 / steps, (time.perf_counter() - t0) / steps


# ---------------------------------------------------------------------------
# the batching workload: eight silicon cells of uneven size
# ---------------------------------------------------------------------------
A_SI = 10.26
_DIAMOND = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                     [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])


def diamond_cell(lattice) -> np.ndarray:
    """Fractional coordinates of the diamond-structure Si atoms inside a cell whose
    lattice vectors (rows) are vectors of the fcc lattice (a = A_SI)."""
    lattice = np.asarray(lattice, dtype=np.float64)
    cart = np.concatenate([(_DIAMOND + np.array(c)) * A_SI
                           for c in itertools.product(range(-3, 4), repeat=3)])
    frac = cart @ np.linalg.inv(lattice)
    keep = np.all((frac > -1e-9) & (frac < 1 - 1e-9), axis=1)
    return np.unique(np.round(frac[keep], 9), axis=0)


def silicon_batch(ecut: float = 8.0, kmesh=(2, 2, 2), sigma_disp: float = 0.03, seed: int = 2024):
    """Si2 (fcc primitive), Si4 (tetragonal a/sqrt2 x a/sqrt2 x a), Si8 x2 (cubic),
    Si16 x2 (1x1x2), Si32 x2 (2x2x1); seeded Gaussian displacements, nband = 2 natom."""
    import addft_gb300 as ad
    a = A_SI
    cells = [0.5 * a * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]]),
             np.array([[a / 2, a / 2, 0], [-a / 2, a / 2, 0], [0, 0, a]]),
             np.eye(3) * a, np.eye(3) * a,
             np.diag([a, a, 2 * a]), np.diag([a, a, 2 * a]),
             np.diag([2 * a, 2 * a, a]), np.diag([2 * a, 2 * a, a])]
    rng = np.random.default_rng(seed)
    out = []
    for lat in cells:
        frac = diamond_cell(lat)
        frac = frac + rng.normal(0, sigma_disp, frac.shape) @ np.linalg.inv(lat)
        out.append(ad.setup(lat, frac, ecut=ecut, nband=2 * frac.shape[0],
                            kmesh=ad.monkhorst_pack(kmesh) if kmesh else None))
    return out
