"""Benchmark: H psi bands/s on the plane-wave microbench, GB300 (sm_103a).

Workload (the H psi / density / XC kernel microbench): cubic box 72^3 with
a = 36 Bohr, G-sphere of radius 0.45*72 (nG = 142,609), 64 bands of i.i.d.
complex normal coefficients (seeded) orthonormalised by Cholesky-QR,
V_loc(r) = sum of 16 real plane waves with amplitudes U(0, 0.5) Ha, 8 atoms
at random fractional positions x 4 projectors (l = 0 and l = 1 x 3) with
beta_l(G) = |G|^l exp(-|G|^2/2), D = diag(1 Ha).  One step = one FP32
application of H = T + V_loc + V_NL to all 64 bands.

The line also carries ``batch8``: H psi of every band and k point of eight
silicon cells of uneven size (2x2x2 k mesh, ecut 8) as one captured CUDA graph
with autotuned per-box launch shapes, against eager launches (``--batch 0``
skips it), and ``si64_scf_force_stress``: wall time of a full SCF +
free energy + forces + stress on Si64 (64 atoms, ecut 15 Ha, 160 bands) with
FP32 H psi and FP64 refinement against the plain FP64 kernel form, and the
energy / force / stress differences between the two, with ``subspace_gemm``:
the refinement's FP64 subspace products in double-float arithmetic against
cuBLAS ZGEMM on the Si64 shapes (``--scf 0`` skips both).

Prints one JSON line.  ``--impl reference`` times the reference algorithm on
the host cores instead (the NumPy/SciPy port in oracle/, all host threads;
the reference's JAX path cannot be installed offline).  Under torchrun each
rank runs an independent replica on its own GPU (the H psi of independent
structures / k points does not exchange data); value = all ranks' bands / max
rank time.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "ad-dft_gb300"))

BOX = 72
NBANDS = 64
NATOM = 8
NPW = 16
SEED = 20261203
METRIC = "H psi bands/s (FP32 H psi, microbench 72^3 box, 64 bands, 8 atoms x 4 projectors)"
WORKLOAD = ("H psi microbench: 72^3 FFT box, a = 36 Bohr, G-sphere radius 0.45*72 (nG 142609), "
            "64 orthonormal bands, V_loc = 16 plane waves, 8 atoms x 4 projectors (l=0,1), D = 1 Ha")


def sphere_miller(n, frac_radius=0.45):
    r = int(np.floor(frac_radius * n))
    m = np.stack(np.meshgrid(*(np.arange(-r, r + 1),) * 3, indexing="ij"), -1).reshape(-1, 3)
    m = m[np.sum(m * m, axis=1) <= (frac_radius * n) ** 2]
    order = np.lexsort((m[:, 2], m[:, 1], m[:, 0], np.sum(m * m, axis=1)))
    return np.ascontiguousarray(m[order].astype(np.int32))


def host_workload(n=BOX, nb=NBANDS, seed=SEED):
    """Seeded host inputs shared by both arms."""
    rng = np.random.default_rng(seed)
    miller = sphere_miller(n)
    nG = miller.shape[0]
    lat = np.eye(3) * (0.5 * n)
    psi = rng.normal(size=(nb, nG)) + 1j * rng.normal(size=(nb, nG))
    # Cholesky-QR orthonormalisation in FP64
    S = psi.conj() @ psi.T
    L = np.linalg.cholesky(S)
    psi = np.linalg.solve(L, psi)
    # V_loc(r): 16 real plane waves inside the sphere, amplitudes U(0, 0.5) Ha
    idx = np.stack(np.meshgrid(*(np.arange(n),) * 3, indexing="ij"), -1).reshape(-1, 3) / n
    v = np.zeros(n ** 3)
    pick = miller[rng.integers(1, nG, NPW)]
    for mvec, amp, ph in zip(pick, rng.uniform(0, 0.5, NPW), rng.uniform(0, 2 * np.pi, NPW)):
        v += amp * np.cos(2 * np.pi * (idx @ mvec) + ph)
    pos = rng.uniform(0, 1, (NATOM, 3)) @ lat
    return dict(n=n, nb=nb, miller=miller, nG=nG, lat=lat, psi=psi, v=v, pos=pos)


def model(nG, N, nb, P, c=8, r=4):
    """Algorithmic bytes / flops of one H psi application (compulsory traffic, textbook FLOPs)."""
    byts = 2 * c * nG * nb + r * N + 4 * nG + c * P * nG + 8 * P * P
    fft_flops = 2 * 5 * N * np.log2(N) * nb
    proj_flops = 16 * P * nG * nb
    return float(byts), float(fft_flops), float(proj_flops)


# ---------------------------------------------------------------------------
# clocks sampling (nvidia-smi, 200 ms) during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = np.array([float(r[1]) for r in rows])
        smax = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[5 + j].strip().lower() == "active"})
        load = sm[sm > 0.5 * smax] if np.any(sm > 0.5 * smax) else sm
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": smax, "reasons": reasons,
                "samples": int(len(rows)), "power_w_max": float(max(float(r[3]) for r in rows))}


# ---------------------------------------------------------------------------
# reference / CPU arm
# ---------------------------------------------------------------------------
def cpu_hpsi_rate(wl, tables, seconds=10.0, sample_bands=4, max_reps=1000, workers=None):
    from oracle import pw  # the checker, used here only as the CPU baseline
    workers = workers or os.cpu_count()
    kin, proj, dion = tables
    psi = wl["psi"][:sample_bands]
    shape = (wl["n"],) * 3
    pw.hpsi_tables(shape, wl["miller"], psi, kin, wl["v"], proj, dion, workers=workers)   # warm
    t0 = time.perf_counter()
    reps = 0
    while reps < max_reps and (time.perf_counter() - t0) < seconds:
        pw.hpsi_tables(shape, wl["miller"], psi, kin, wl["v"], proj, dion, workers=workers)
        reps += 1
    dt = time.perf_counter() - t0
    return sample_bands * reps / dt, workers, f"{reps} x H psi on {sample_bands} of the 64 bands, {dt:.1f} s"


def host_tables(wl):
    """Kinetic, projector and D tables on the host, built with the oracle (reference formulas)."""
    from oracle import pw
    lat, miller = wl["lat"], wl["miller"]
    g = miller @ pw.reciprocal(lat)
    kin = 0.5 * np.sum(g * g, axis=1)
    psp = pw.Pseudo(proj_w=(1.0, 1.0), proj_b=(1.0, 1.0), proj_l=(0, 1), dion=np.eye(2))
    basis = pw.Basis(miller=miller, ecut=0.0, fft_shape=(wl["n"],) * 3, miller_rho=miller)
    st = pw.Static(basis=basis, kpts=np.zeros((1, 3)), kweights=np.ones(1), psp=psp, natom=NATOM, nband=NBANDS,
                   spin_degeneracy=2.0, sigma=0.05, nelec=0.0, eta_ewald=0.9)
    proj = pw.projectors(st, lat, wl["pos"] @ np.linalg.inv(lat))[0]
    dion = pw.dion_full(psp, NATOM)
    return kin, proj, dion


def run_reference(args, rank, world):
    """The reference algorithm on the host cores: each step is H psi on a bounded band sample."""
    if rank != 0:
        return
    from oracle import pw  # the CPU implementation being timed (NumPy/SciPy port)
    wl = host_workload()
    kin, proj, dion = host_tables(wl)
    workers = os.cpu_count()
    sample = 4
    psi = wl["psi"][:sample]
    shape = (wl["n"],) * 3

    def step():
        pw.hpsi_tables(shape, wl["miller"], psi, kin, wl["v"], proj, dion, workers=workers)

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    total = float(np.sum(times))
    value = sample * args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "bands/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "sample": f"{sample} of the 64 bands per step"},
            "cpu_baseline": {"value": value, "unit": "bands/s", "cores": workers, "kind": "port",
                             "sample": f"H psi on {sample} of the 64 bands per step, {args.steps} steps "
                                       "(NumPy/SciPy port of the reference algorithm, scipy.fft workers = all "
                                       "host cores; the reference's JAX path is not installable offline)"},
            "e2e": {"value": value, "unit": "bands/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Si64 SCF + forces + stress: FP32 H psi with FP64 refinement vs plain FP64
# ---------------------------------------------------------------------------
SI64 = ("Si64: 2x2x2 diamond supercell, a = 20.52 Bohr, seeded displacements sigma = 0.05 Bohr, "
        "ecut 15 Ha, Gamma only, 160 bands, synthetic Si-like norm-conserving pseudopotential, LDA-PZ, "
        "SCF to a density residual of 1e-10, then free energy, forces and stress")


def si64_system():
    import addft_gb300 as ad
    a = 10.26
    base = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                     [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
    cells = [(i, j, k) for i in range(2) for j in range(2) for k in range(2)]
    frac = np.concatenate([(base + np.array(c)) / 2.0 for c in cells])
    lat = np.eye(3) * 2 * a
    frac = frac + np.random.default_rng(64).normal(0, 0.05, frac.shape) / (2 * a)
    return ad.setup(lat, frac, ecut=15.0, nband=160)


def scf_force_block():
    """Wall time of SCF + free energy + forces + stress on Si64 in both precisions
    (after a warm-up of both paths), and the FP32+refine errors against FP64."""
    import torch
    from addft_gb300 import observables as obs, solver
    from addft_gb300.geometry import volume
    from addft_gb300.system import build_geometry_cache

    s = si64_system()
    geo, st = s.geo, s.static

    def run(prec, **kw):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cache = build_geometry_cache(geo, st)
        state = solver.solve_scf(geo, st, cache=cache, precision=prec, **kw)
        e = obs.mermin_free_energy(geo, st, state, cache)
        dR, deps = obs.envelope_gradients(geo, st, state, cache, precision=prec)
        f = obs.forces_from_dR(dR)
        sig = obs.stress_from_deps(volume(geo.lattice), deps)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, e, f, sig, int(state.n_iter), float(state.residual)

    # warm-up: one full untimed run of each arm (library handles and workspaces for every
    # subspace size the run meets, allocator pools, plans, gradient kernels)
    run("fp32")
    run("fp64")
    t32, e32, f32, s32, it32, r32 = run("fp32")
    t64, e64, f64, s64, it64, r64 = run("fp64")
    return {"workload": SI64, "fp32_refine_s": t32, "fp64_s": t64, "speedup": t64 / t32,
            "dE_per_atom_ha": abs(e32 - e64) / st.natom, "max_dforce_ha_bohr": float(np.max(np.abs(f32 - f64))),
            "max_dstress_ha_bohr3": float(np.max(np.abs(s32 - s64))), "energy_ha": e64,
            "scf_iterations": {"fp32_refine": it32, "fp64": it64}, "residual": {"fp32_refine": r32, "fp64": r64},
            "timed": "structure cache, SCF (incl. 4 polish steps), free energy, forces, stress; "
                     "basis setup excluded; both arms warmed up by one full untimed run each"}


def si64_kernel_breakdown(top=30):
    """GPU time per operator / kernel of one FP32+refine Si64 SCF + forces + stress run (after a
    warm-up run), from torch.profiler (CUPTI): where the FP32 arm's wall time goes.  Printed as
    text lines; not part of the bench line (a run under the profiler is slower)."""
    import torch
    from torch.profiler import ProfilerActivity, profile
    from addft_gb300 import observables as obs, solver
    from addft_gb300.geometry import volume
    from addft_gb300.system import build_geometry_cache
    s = si64_system()
    geo, st = s.geo, s.static

    def run():
        cache = build_geometry_cache(geo, st)
        state = solver.solve_scf(geo, st, cache=cache, precision="fp32")
        obs.mermin_free_energy(geo, st, state, cache)
        dR, deps = obs.envelope_gradients(geo, st, state, cache, precision="fp32")
        obs.stress_from_deps(volume(geo.lattice), deps)
        torch.cuda.synchronize()

    run()
    with profile(activities=[ProfilerActivity.CPU, ProfilerActivity.CUDA]) as prof:
        run()
    rows = []
    for e in prof.key_averages():
        t = getattr(e, "device_time_total", None) or getattr(e, "cuda_time_total", 0)
        rows.append((t, e.count, e.key))
    rows.sort(reverse=True)
    for t, n, key in rows[:top]:
        print(f"{t / 1e3:10.1f} ms  calls {n:6d}  {key[:110]}", flush=True)


def subspace_gemm_block(reps=10):
    """The refinement's FP64 subspace products on the Si64 shapes (168 bands + blocks,
    nG 23,847): double-float GEMM on the FP32 pipes against cuBLAS FP64 ZGEMM (CUDA
    events; max error relative to |op(a)| |op(b)|)."""
    import torch
    from addft_gb300 import ops
    g = torch.Generator(device="cuda").manual_seed(SEED)

    def rnd(*shape):
        return torch.complex(torch.randn(*shape, generator=g, device="cuda", dtype=torch.float64),
                             torch.randn(*shape, generator=g, device="cuda", dtype=torch.float64))

    def timed_ms(f):
        f()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        for _ in range(reps):
            f()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    out = {}
    x, y, u, z = rnd(168, 23847), rnd(336, 23847), rnd(168, 168).transpose(0, 1), rnd(168, 23847)
    cases = {"projection conj(X) Y^T 168x336x23847": (x, y.transpose(0, 1), True, False),
             "rotation U X 168x23847x168": (u, z, False, False)}
    for name, (a, b, ca, cb) in cases.items():
        M, K = a.shape
        N = b.shape[1]
        ref = (a.conj() if ca else a) @ (b.conj() if cb else b)
        err = float((ops.zgemm_df(a, b, ca, cb) - ref).abs().max() / (a.abs() @ b.abs()).max())
        td = timed_ms(lambda: ops.zgemm_df(a, b, ca, cb))
        tc = timed_ms(lambda: (a.conj() if ca else a) @ (b.conj() if cb else b))
        fl = 8.0 * M * N * K
        out[name] = {"double_float_ms": td, "double_float_tflops": fl / td / 1e9, "zgemm_fp64_ms": tc,
                     "zgemm_fp64_tflops": fl / tc / 1e9, "rel_err": err}
    return out


# ---------------------------------------------------------------------------
# batch of eight structures: one captured graph, autotuned launch shapes
# ---------------------------------------------------------------------------
BATCH = ("8 silicon cells (Si2 fcc, Si4 tetragonal, Si8 x2, Si16 x2, Si32 x2; seeded 0.03 Bohr "
         "displacements), 2x2x2 Monkhorst-Pack, ecut 8 Ha, nband = 2 natom, FFT boxes 24^3 .. 60x60x30; "
         "one step = FP32 H psi of every band and k point of all eight (1888 band-k)")


def batch_block(steps=20):
    import torch
    from addft_gb300._lib import LIB
    from addft_gb300.batch import HpsiBatch, items_from_systems, silicon_batch, timed

    systems = silicon_batch()
    b = HpsiBatch(items_from_systems(systems))
    t_default, _ = timed(b.run_eager, steps)
    tunings = b.tune()
    t_eager, w_eager = timed(b.run_eager, steps)
    l0 = LIB.addft_launch_count()
    b.run_eager()                                  # the launch sequence the graph records
    torch.cuda.synchronize()
    launches = LIB.addft_launch_count() - l0
    b.capture(branches=1)
    t_graph1, _ = timed(b.run, steps)
    b.capture(branches=4)
    t_graph, w_graph = timed(b.run, steps)
    return {"workload": BATCH, "bands_per_step": b.bands,
            "graph": {"value": b.bands / t_graph, "unit": "band-k/s", "ms_per_step": 1e3 * t_graph,
                      "host_ms_per_step": 1e3 * w_graph, "branches": 4},
            "graph_one_branch": {"value": b.bands / t_graph1, "ms_per_step": 1e3 * t_graph1},
            "eager_tuned": {"value": b.bands / t_eager, "ms_per_step": 1e3 * t_eager,
                            "host_ms_per_step": 1e3 * w_eager},
            "eager_default_tuning": {"value": b.bands / t_default, "ms_per_step": 1e3 * t_default},
            "tuning": [{"box": list(it.plan.shape), **it.tuning} for it in b.items],
            "kernel_launches_in_graph": int(launches)}


# ---------------------------------------------------------------------------
# arithmetic peaks of this GPU (compute-roof denominators)
# ---------------------------------------------------------------------------
PEAK_RUNS = (("fp32_fma", 0, 1_000_000), ("fp64_fma", 1, 20_000), ("tf32_mma_sync", 2, 600_000),
             ("tf32_tcgen05", 3, 4_000_000))


def measure_peaks(dev):
    """FP32 FMA, FP64 FMA, TF32 mma.sync and TF32 tcgen05 rates from kernels that do
    nothing else (addft_peak_flops, up to about a second each, CUDA events), with the SM
    clocks sampled while they run."""
    import ctypes as C
    import torch
    from addft_gb300._lib import LIB, check
    sink = torch.empty(1 << 20, dtype=torch.uint8, device=dev)
    out = {}
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    with ClockSampler(dev.index) as clk:
        for key, which, iters in PEAK_RUNS:
            tf, ms = C.c_double(), C.c_float()
            check(LIB.addft_peak_flops(which, iters, C.byref(tf), C.byref(ms), C.c_void_p(sink.data_ptr()), stream),
                  "peak_flops")
            out[key] = {"tflops": tf.value, "ms": ms.value, "iters": iters}
    out["clocks"] = clk.summary()
    return out


# ---------------------------------------------------------------------------
# replicas: one independent H psi per rank, max-over-ranks timing
# ---------------------------------------------------------------------------
def max_over_ranks(t: float, world: int, device="cpu") -> float:
    """Slowest rank's time (all_reduce MAX); the identity on one rank."""
    if world <= 1:
        return float(t)
    import torch
    import torch.distributed as dist
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt)


def replica_value(bands_per_step: int, steps: int, t_max: float, world: int) -> float:
    """Whole-job throughput: every rank's bands over the slowest rank's time (weak scaling)."""
    return world * bands_per_step * steps / t_max


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args, rank, world):
    import torch
    import torch.distributed as dist

    from addft_gb300 import ops
    from addft_gb300._lib import LIB
    from addft_gb300.geometry import reciprocal, volume
    from addft_gb300.psp import Pseudo

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    wl = host_workload(n=args.box, nb=args.nbands)
    n, nb, nG, lat = wl["n"], wl["nb"], wl["nG"], wl["lat"]
    N = n ** 3
    plan = ops.Plan((n, n, n), wl["miller"])
    bv, om = reciprocal(lat), volume(lat)
    psp = Pseudo(proj_w=(1.0, 1.0), proj_b=(1.0, 1.0), proj_l=(0, 1), dion=np.eye(2))
    P = NATOM * psp.nh
    psi32 = torch.as_tensor(wl["psi"], device=dev).to(torch.complex64).reshape(1, nb, nG).contiguous()
    kin32 = ops.kinetic(plan, bv, np.zeros((1, 3)), dtype=torch.float32)
    v32 = torch.as_tensor(wl["v"], device=dev).to(torch.float32)
    proj32 = ops.projectors(plan, bv, om, np.zeros((1, 3)), wl["pos"], psp, dtype=torch.complex64)
    dion32 = torch.eye(P, dtype=torch.float32, device=dev)
    out = torch.empty_like(psi32)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2

    def step():
        ops.hpsi(plan, psi32, kin32, v32, proj32, dion32, out=out)

    # correctness guard on the timed path: FP32 vs FP64 of the same inputs
    psi64 = psi32.to(torch.complex128)
    ref = ops.hpsi(plan, psi64, kin32.double(), v32.double(), proj32.to(torch.complex128), dion32.double())
    step()
    err = float((out.to(torch.complex128) - ref).abs().max() / ref.abs().max())
    assert err < 1e-5, f"FP32 H psi deviates from FP64 by {err:.2e}"

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = LIB.addft_launch_count()
    with ClockSampler(dev.index) as clk:
        for s, e in ev:
            flush.zero_()                     # evict L2 between timed steps (not timed)
            s.record()
            step()
            e.record()
        torch.cuda.synchronize()
    launches = LIB.addft_launch_count() - l0
    ms = [s.elapsed_time(e) for s, e in ev]
    t_total = max_over_ranks(sum(ms) / 1e3, world, dev)
    value = replica_value(nb, args.steps, t_total, world)
    t_launch = t_total / args.steps

    # e2e through the C ABI with pinned host buffers: addft_hpsi_host uploads psi, applies H and
    # downloads the result every step, in band chunks whose copies overlap the compute
    h_in = torch.empty((1, nb, nG), dtype=torch.complex64, pin_memory=True)
    h_in.copy_(psi32.cpu())
    h_out = torch.empty_like(h_in, pin_memory=True)

    def e2e_step():
        ops.hpsi_host(plan, h_in, kin32, v32, proj32, dion32, out_h=h_out, chunk_bands=args.e2e_chunk)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s, e in ev2:
        flush.zero_()
        s.record()
        e2e_step()
        e.record()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(sum(s.elapsed_time(e) for s, e in ev2) / 1e3, world, dev)
    e2e = replica_value(nb, args.steps, t_e2e, world)
    nbytes = psi32.numel() * 8

    # the plain FP64 kernel form of the same step (for the FP32-vs-FP64 ratio)
    kin64, v64 = kin32.double(), v32.double()
    proj64, dion64 = proj32.to(torch.complex128), dion32.double()
    out64 = torch.empty_like(psi64)
    for _ in range(2):
        ops.hpsi(plan, psi64, kin64, v64, proj64, dion64, out=out64)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(3):
        ops.hpsi(plan, psi64, kin64, v64, proj64, dion64, out=out64)
    e.record()
    torch.cuda.synchronize()
    t64 = s.elapsed_time(e) / 3e3

    if rank != 0:
        return
    mpeaks = measure_peaks(dev) if args.peaks else None
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    byts, fft_f, proj_f = model(nG, N, nb, P)
    achieved = byts / t_launch / 1e9
    # arithmetic roof: FFT flops at the FP32 FMA rate plus projector flops at the rates of the
    # kernels that run them -- half the projector flops are becp (split-TF32 mma.sync), half
    # the V_NL apply (split-TF32 tcgen05), three MMAs per product -- all measured on this GPU
    # by measure_peaks (nominal rates if --peaks 0)
    fp32_peak = 152 * 128 * 2 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    tf32_peak, tc05_peak = 1100.0, 1100.0
    peak_kind = "nominal"
    if mpeaks:
        fp32_peak = mpeaks["fp32_fma"]["tflops"]
        tf32_peak = mpeaks["tf32_mma_sync"]["tflops"]
        tc05_peak = mpeaks["tf32_tcgen05"]["tflops"]
        peak_kind = "measured (addft_peak_flops on this GPU)"
    becp_rate = tf32_peak / 3.0 if os.environ.get("ADDFT_BECP_TC", "1") == "1" else fp32_peak
    apply_rate = tc05_peak / 3.0 if os.environ.get("ADDFT_APPLY_TC", "3") == "3" else tf32_peak / 3.0
    t_hbm, t_fp32 = byts / (hbm * 1e9), fft_f / (fp32_peak * 1e12)
    t_tc = 0.5 * proj_f / (becp_rate * 1e12) + 0.5 * proj_f / (apply_rate * 1e12)
    proj_peak = proj_f / t_tc / 1e12
    traffic = None
    tf = ROOT / "profiles" / "hpsi_microbench72_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("dram_bytes_per_hpsi")
    if args.cpu_seconds > 0:
        cb_value, cores, sample = cpu_hpsi_rate(wl, host_tables(wl), seconds=args.cpu_seconds)
    else:
        cb_value, cores, sample = None, 0, "skipped (--cpu-seconds 0)"
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "bands/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_launch, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "parallelism": f"replicas x{world}", "l2": "flushed between steps",
                   "precision": "FP32 H psi (FFT, V(r) psi, projector GEMMs), FP64 reductions"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "of": "measured MEASURED_PEAKS.json hbm_gbs",
                     "kernel": "one addft_hpsi call (z-column inverse, xy-plane FFT with V(r), z-column forward "
                               "+ kinetic; becp / split sums / D becp on a forked stream; V_NL apply on tcgen05)",
                     "algorithmic_bytes_per_launch": byts,
                     "fft_tflops": fft_f / t_launch / 1e12, "projector_tflops": proj_f / t_launch / 1e12,
                     "compute_roof": {"fp32_tflops": fp32_peak, "tf32_mma_sync_tflops": tf32_peak,
                                      "tf32_tcgen05_tflops": tc05_peak,
                                      "projector_rate_tflops": proj_peak, "peaks": peak_kind,
                                      "t_hbm_us": 1e6 * t_hbm, "t_fp32_fft_us": 1e6 * t_fp32,
                                      "t_projector_us": 1e6 * t_tc,
                                      "binds": "fp32_fft+tc" if t_fp32 + t_tc > t_hbm else "hbm",
                                      "frac": max(t_hbm, t_fp32 + t_tc) / t_launch}},
        "cpu_baseline": {"value": cb_value, "unit": "bands/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": e2e, "unit": "bands/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "call": f"addft_hpsi_host, pinned host psi in and H psi out, chunks of {args.e2e_chunk} bands "
                        "with upload / H psi / download overlapped"},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "fp64_hpsi": {"value": nb / t64, "unit": "bands/s", "ms_per_step": 1e3 * t64,
                      "fp32_over_fp64": t64 / t_launch},
        "fp32_vs_fp64_rel_err": err,
        "measured_peaks": mpeaks,
    }
    if args.batch:
        line["batch8"] = batch_block()
    if args.scf:
        line["subspace_gemm"] = subspace_gemm_block()
        line["si64_scf_force_stress"] = scf_force_block()
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--box", type=int, default=BOX, help="FFT box edge (profiling cases use smaller boxes)")
    ap.add_argument("--nbands", type=int, default=NBANDS)
    ap.add_argument("--scf", type=int, default=1, help="1: add the Si64 SCF+forces FP32+refine vs FP64 block")
    ap.add_argument("--batch", type=int, default=1, help="1: add the 8-structure graph-captured batch block")
    ap.add_argument("--peaks", type=int, default=1, help="1: measure FP32/FP64/TF32 peaks for the compute roof")
    ap.add_argument("--e2e-chunk", type=int, default=32, help="bands per chunk of the host-buffer (e2e) H psi")
    ap.add_argument("--si64-breakdown", type=int, default=0,
                    help="1: only print the GPU time per kernel of one FP32+refine Si64 run (torch.profiler)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.si64_breakdown:
        return si64_kernel_breakdown()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    try:
        run_gpu(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
