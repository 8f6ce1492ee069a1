"""Golden values computed by the REFERENCE's own code on the fixture systems.

The reference is JAX code and JAX is not installed here, so this script runs it on
NumPy through the value-only stand-in in ``refshim/`` (``jax.numpy`` -> NumPy, eager
``jit`` / ``lax`` loops, and ``jax.grad`` by complex steps, which the reference's SCF
uses only for the PZ81 XC potential, a real-analytic function of the density).  The
reference sources are read where they lie; nothing of them is copied.  The native
kernels are off (``ADDFT_NATIVE_PACK=0``, no FFI), the XC is the analytic PZ81
(``ADDFT_XC=analytic``, libxc is absent).

Per system it records the SCF (iterations, residual, eigenvalues, occupations, mu,
the density on the FFT grid), the Mermin free energy (``addft.energy``), the seven
energy terms (``addft.energy_decomposition``), and the forces and stress as central
differences of the reference's own free energy over full SCF runs (Richardson
extrapolation of h = 1e-3 and 5e-4, Bohr for displacements, dimensionless for strain)
-- the reference's own forces and stress come from ``jax.grad`` through FFTs, which
complex steps cannot replace.

The same SCF quantities for the differentiation workload (Si8, ecut 10, 20 bands), where
one complex step per grid point would be too slow: there the XC potential is the same
derivative taken point by point (``_pointwise_xc_potential``, checked against the
per-component path on the fixture box before use).  And for the fixture cell with the
UPF test pseudopotentials
(s/p channels, and with an added d channel) read by the reference's own UPF reader.
It also records the reference's Delta Q observable on the fixture cell with its
position derivative by central differences over full SCF runs, building blocks on
the Si8 cell (Ewald energy with
central-difference derivatives, local and Hartree potentials, occupations), the
reference's basis builder (Miller sets in their frozen order, FFT
boxes) and Monkhorst-Pack meshes on the host-test cells, reads the UPF test files with
the reference's reader and samples its radial
transforms (beta_q, vloc_q) on a q grid, builds the Systems the reference's ABACUS
adapter makes of the case
directories tests/test_abacus_case.py writes, and runs the reference's H psi (ops/hpsi.py) and band density (physics/density.py)
on the H psi microbench's seeded workload at 15^3, 48^3 and 72^3 (2 bands), stored as
sampled entries and seeded random projections (``micro_checks``).

Run from the repository root, in a container that has the reference at
/root/reference:  ``python tests/golden/make_reference_fixtures.py [--micro-only | --stress-only | --upf-only | --si8-only | --abacus-only |
--upf-reader-only | --basis-only | --physics-only | --dq-only | --system NAME]``
Writes tests/golden/ref_fixtures.json.
"""

from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE_SRC = Path("/root/reference/src")

SYSTEMS = {
    # the reference's tests/conftest.py fixture cell (6 Bohr cubic, distorted pair)
    "si2_gamma": dict(lattice=np.eye(3) * 6.0, frac=[[0.0, 0.0, 0.0], [0.53, 0.47, 0.49]], ecut=2.0, nband=2,
                      density_factor=4.0, kmesh=None, forces=True),
    # the same cell on a 2x2x2 Monkhorst-Pack mesh
    "si2_mp222": dict(lattice=np.eye(3) * 6.0, frac=[[0.0, 0.0, 0.0], [0.53, 0.47, 0.49]], ecut=2.0, nband=2,
                      density_factor=4.0, kmesh=(2, 2, 2), forces=True),
    # a denser basis on the Gamma point (nG larger than the box rule's minimum)
    "si2_gamma_ecut4": dict(lattice=np.eye(3) * 6.0, frac=[[0.0, 0.0, 0.0], [0.53, 0.47, 0.49]], ecut=4.0,
                            nband=4, density_factor=4.0, kmesh=None, forces=False),
}
# the fixture cell with the UPF test pseudopotentials (tests/golden/make_test_upf.py): s/p
# channels (v2 format) and with an added l = 2 channel
UPF_SYSTEMS = {
    "si2_upf_v2": dict(lattice=np.eye(3) * 6.0, frac=[[0.0, 0.0, 0.0], [0.53, 0.47, 0.49]], ecut=3.0, nband=6,
                       density_factor=4.0, kmesh=None, forces=False, upf="si_test_v2.upf"),
    "si2_upf_d": dict(lattice=np.eye(3) * 6.0, frac=[[0.0, 0.0, 0.0], [0.53, 0.47, 0.49]], ecut=3.0, nband=6,
                      density_factor=4.0, kmesh=None, forces=False, upf="si_test_d_v2.upf"),
}
H_FD = (1e-3, 5e-4)


# the differentiation workload: Si8 conventional diamond cell, a = 10.26 Bohr, seeded 0.05 Bohr
# displacements (seed 8), ecut 10 Ha, Gamma, 20 bands
_A8 = 10.26
_BASE8 = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                   [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
SI8_SYSTEMS = {
    "si8_ecut10": dict(lattice=np.eye(3) * _A8,
                       frac=(_BASE8 + np.random.default_rng(8).normal(0, 0.05, _BASE8.shape) / _A8).tolist(),
                       ecut=10.0, nband=20, density_factor=4.0, kmesh=None, forces=False),
}


def _pointwise_xc_potential(xc):
    """The reference's v_xc = (N / Omega) jax.grad(E_xc) for its LDA energy
    E_xc = (Omega / N) sum_j e(n_j) (xc_energy_lda, a sum of point terms): the gradient is
    e'(n_j) point by point, taken here by one complex step of the reference's own point
    function e = lda_energy_density over the whole grid, instead of one complex step per
    grid point -- the same values at the cost of one evaluation."""
    h = 1e-30

    def xc_potential_r(xc_energy_fn, basis, lattice, rho_r):
        assert xc_energy_fn is xc.xc_energy_lda
        rho = np.asarray(rho_r, dtype=np.float64)
        return np.asarray(np.imag(xc.lda_energy_density(rho + 1j * h)) / h).view(type(rho_r))
    return xc_potential_r


def _reference(pointwise_xc=False):
    os.environ["ADDFT_XC"] = "analytic"
    os.environ["ADDFT_NATIVE_PACK"] = "0"
    for p in (str(REFERENCE_SRC), str(HERE / "refshim")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import addft
    assert Path(addft.__file__).resolve().is_relative_to(REFERENCE_SRC), addft.__file__
    if pointwise_xc:
        from addft.geometry.cell import volume
        from addft.physics import xc
        fast = _pointwise_xc_potential(xc)
        # the substitute equals the reference's own path: check on a random density of the fixture box
        s = addft.setup(np.eye(3) * 6.0, [[0, 0, 0], [0.53, 0.47, 0.49]], ecut=2.0, nband=2)
        rho = np.random.default_rng(3).uniform(0.01, 0.2, int(np.prod(s.static.basis.fft_shape)))
        ref = xc.xc_potential_r(xc.xc_energy_lda, s.static.basis, s.geo.lattice, rho)
        got = fast(xc.xc_energy_lda, s.static.basis, s.geo.lattice, rho)
        assert np.max(np.abs(np.asarray(ref) - np.asarray(got))) < 1e-13 * np.max(np.abs(ref))
        e = xc.xc_energy_lda(s.static.basis, s.geo.lattice, rho)
        assert abs(e - float(volume(s.geo.lattice)) / rho.size * np.sum(xc.lda_energy_density(rho))) < 1e-12
        xc.xc_potential_r = fast
    return addft


def _setup(ad, spec, frac=None):
    kmesh = ad.monkhorst_pack(spec["kmesh"]) if spec["kmesh"] else None
    psp = ad.geometry.psp.from_upf(str(HERE / spec["upf"])) if spec.get("upf") else None
    return ad.setup(spec["lattice"], spec["frac"] if frac is None else frac, psp=psp, ecut=spec["ecut"],
                    nband=spec["nband"], density_factor=spec["density_factor"], kmesh=kmesh)


def _free_energy(ad, spec, frac):
    s = _setup(ad, spec, frac)
    return float(ad.energy(s, ad.scf(s)))


RHO_FULL_MAX = 5000   # densities on larger boxes are stored as checks, not in full


def rho_checks(rho):
    idx, smp, prj = micro_checks(np.asarray(rho)[None])
    return {"idx": idx.tolist(), "samples": smp[0].tolist(), "proj": _c(prj[0]), "sum": float(np.sum(rho))}


def run_system(ad, name, spec):
    t0 = time.time()
    s = _setup(ad, spec)
    st = ad.scf(s)
    e = float(ad.energy(s, st))
    terms = {k: float(v) for k, v in ad.energy_decomposition(s, st).items()}
    out = {
        "lattice": np.asarray(spec["lattice"]).tolist(), "frac": np.asarray(spec["frac"]).tolist(),
        "ecut": spec["ecut"], "nband": spec["nband"], "density_factor": spec["density_factor"],
        "kmesh": spec["kmesh"], "upf": spec.get("upf"), "nG": int(np.asarray(s.static.basis.miller).shape[0]),
        "fft_shape": [int(x) for x in s.static.basis.fft_shape],
        "free_energy": e, "terms": terms, "n_iter": int(st.n_iter), "residual": float(st.residual),
        "eig": np.asarray(st.eig).tolist(), "occ": np.asarray(st.occ).tolist(), "mu": float(st.mu),
    }
    rho = np.asarray(st.rho_r)
    if rho.size <= RHO_FULL_MAX:
        out["rho_r"] = rho.tolist()
    else:   # large boxes: sampled entries, seeded projections and the sum (micro_checks)
        out["rho_checks"] = rho_checks(rho)
    if spec["forces"]:
        frac0 = np.asarray(spec["frac"], dtype=float)
        lat = np.asarray(spec["lattice"], dtype=float)
        inv = np.linalg.inv(lat)
        f = np.zeros_like(frac0)
        for a in range(frac0.shape[0]):
            for c in range(3):
                d = []
                for h in H_FD:
                    step = np.zeros(3)
                    step[c] = h
                    fp, fm = frac0.copy(), frac0.copy()
                    fp[a] += step @ inv
                    fm[a] -= step @ inv
                    d.append((_free_energy(ad, spec, fp) - _free_energy(ad, spec, fm)) / (2 * h))
                # error of the central difference is c h^2: Richardson with h2 = h1 / 2
                f[a, c] = -(4 * d[1] - d[0]) / 3
        out["forces_fd"] = f.tolist()
        out["forces_fd_h"] = list(H_FD)
        out["stress_fd"] = stress_fd(ad, s).tolist()
    out["seconds"] = time.time() - t0
    return out


def stress_fd(ad, s):
    """sigma = -(1/Omega) dF/deps (symmetric strain, the basis held fixed as the reference's
    make_energy(static) does) by central differences of the reference's free energy,
    Richardson-extrapolated over H_FD."""
    from addft.geometry.cell import strained, volume
    e_fn = ad.make_energy(s.static)
    omega = float(volume(s.geo.lattice))
    sig = np.zeros((3, 3))
    for i in range(3):
        for j in range(i, 3):
            d = []
            for h in H_FD:
                eps = np.zeros((3, 3))
                eps[i, j] += 0.5 * h
                eps[j, i] += 0.5 * h
                fp = float(e_fn(strained(s.geo, eps)))
                fm = float(e_fn(strained(s.geo, -eps)))
                d.append((fp - fm) / (2 * h))
            sig[i, j] = sig[j, i] = -((4 * d[1] - d[0]) / 3) / omega
    return sig


# H psi / density microbench (bench.py's seeded workload: sphere of radius 0.45 n, orthonormal
# bands, V_loc of 16 plane waves, 8 atoms x 4 projectors with beta_l = |G|^l exp(-|G|^2 / 2),
# D = 1 Ha) on the reference's ops/hpsi.py and physics/density.py.  The outputs are stored as
# size-independent checks: 64 sampled entries per band and 4 seeded random projections.
MICRO_BOXES = (15, 48, 72)
MICRO_BANDS = 2
N_SAMPLES, N_PROJ, CHECK_SEED = 64, 4, 7


def micro_checks(x, seed=CHECK_SEED):
    """Sampled entries and seeded random projections of a (nb, n) array (also used by the tests)."""
    x = np.asarray(x).reshape(x.shape[0], -1)
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(x.shape[1], size=min(N_SAMPLES, x.shape[1]), replace=False))
    w = rng.normal(size=(N_PROJ, x.shape[1])) + 1j * rng.normal(size=(N_PROJ, x.shape[1]))
    proj = x @ w.T                                    # (nb, N_PROJ)
    return idx, x[:, idx], proj


def _c(z):
    z = np.asarray(z)
    return {"re": z.real.tolist(), "im": z.imag.tolist()}


def run_micro(ad, n):
    sys.path.insert(0, str(HERE.parents[1]))
    import bench
    from addft.geometry.basis import Basis
    from addft.geometry.cell import Cell
    from addft.geometry.psp import synthetic
    from addft.ops.hpsi import hpsi
    from addft.physics.density import density_from_psi
    from addft.system import Static
    wl = bench.host_workload(n=n, nb=MICRO_BANDS)
    lat = wl["lat"]
    frac = wl["pos"] @ np.linalg.inv(lat)
    basis = Basis(miller=wl["miller"], ecut=0.0, fft_shape=(n, n, n), miller_rho=wl["miller"])
    psp = synthetic(zval=(4.0,), proj_w=(1.0, 1.0), proj_b=(1.0, 1.0), dion_diag=(1.0, 1.0))
    static = Static(basis=basis, kpts=np.zeros((1, 3)), kweights=np.ones(1), psp=psp,
                    spec_idx=np.zeros(frac.shape[0], dtype=np.int32), nband=MICRO_BANDS, spin_degeneracy=2.0,
                    sigma=0.05, nelec=0.0, eta_ewald=0.9)
    psi = wl["psi"][None]
    h = np.asarray(hpsi(Cell(lattice=lat, frac=frac), static, psi, wl["v"]))[0]
    rho = np.asarray(density_from_psi(basis, lat, psi, np.ones((1, MICRO_BANDS)), np.ones(1), 2.0))
    hi, hs, hp = micro_checks(h)
    ri, rs, rp = micro_checks(rho[None])
    return {"n": n, "nb": MICRO_BANDS, "nG": int(wl["nG"]), "hpsi_idx": hi.tolist(), "hpsi_samples": _c(hs),
            "hpsi_proj": _c(hp), "hpsi_norm": np.linalg.norm(h, axis=1).tolist(),
            "rho_idx": ri.tolist(), "rho_samples": rs[0].tolist(), "rho_proj": _c(rp[0]),
            "rho_sum": float(np.sum(rho))}


UPF_FILES = ("si_test_v1.upf", "si_test_v2.upf", "si_test_d_v2.upf")
Q_GRID = np.linspace(0.0, 8.0, 41)     # 1/Bohr: where the radial transforms are sampled


def _arr_checks(x):
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    w = np.random.default_rng(11).normal(size=x.size)
    return {"size": int(x.size), "sum": float(np.sum(x)), "sumsq": float(np.sum(x * x)), "proj": float(x @ w),
            "head": x[:4].tolist(), "tail": x[-4:].tolist()}


def run_upf(ad):
    """The reference's UPF reader (geometry/upf.py read_upf) on the test files, and its radial
    transforms (geometry/psp.py beta_q / vloc_q of from_upf) on a q grid."""
    from addft.geometry.psp import beta_q, from_upf, vloc_q
    from addft.geometry.upf import read_upf
    out = {}
    for f in UPF_FILES:
        d = read_upf(str(HERE / f))
        psp = from_upf(str(HERE / f))
        rec = {k: (_arr_checks(v) if isinstance(v, np.ndarray) and np.asarray(v).dtype.kind == "f"
                   else np.asarray(v).tolist() if isinstance(v, np.ndarray) else v) for k, v in d.items()}
        rec["beta_q"] = np.asarray(beta_q(psp, 0, Q_GRID)).tolist()
        rec["vloc_q"] = np.asarray(vloc_q(psp, 0, Q_GRID[1:])).tolist()   # q = 0 is a separate limit
        out[f] = rec
    return {"q": Q_GRID.tolist(), "files": out}


# cells of the host basis tests (tests/test_abi_host.py): lattice, ecut, density factor, k mesh
BASIS_CASES = [
    ("cubic6_e2_f4", np.eye(3) * 6.0, 2.0, 4.0, None),
    ("cubic6_e2_f2", np.eye(3) * 6.0, 2.0, 2.0, None),
    ("cubic6_e2_f4_mp222", np.eye(3) * 6.0, 2.0, 4.0, (2, 2, 2)),
    ("si8_e10", np.eye(3) * 10.26, 10.0, 4.0, None),
    ("fcc_e8_mp222", np.array([[0.0, 5.13, 5.13], [5.13, 0.0, 5.13], [5.13, 5.13, 0.0]]), 8.0, 4.0, (2, 2, 2)),
]


def _index_checks(m):
    m = np.asarray(m, dtype=np.int64)
    w = np.arange(1, m.shape[0] + 1, dtype=np.int64)
    return {"n": int(m.shape[0]), "wsum": [int(x) for x in (w[:, None] * m).sum(axis=0)],
            "sq": int(np.sum(m * m)), "head": m[:8].tolist(), "tail": m[-8:].tolist()}


def run_basis(ad):
    """The reference's basis builder (geometry/basis.py make_basis: frozen Miller sets of the
    wavefunction and density shells in their order, FFT box) and Monkhorst-Pack meshes."""
    from addft.geometry.basis import make_basis
    out = {}
    for name, lat, ecut, factor, kmesh in BASIS_CASES:
        km = ad.monkhorst_pack(kmesh) if kmesh else ad.gamma()
        kc = np.asarray(km.cartesian(lat))
        b = make_basis(lat, ecut, factor, kpts=kc)
        out[name] = {"lattice": np.asarray(lat).tolist(), "ecut": ecut, "density_factor": factor, "kmesh": kmesh,
                     "kfrac": np.asarray(km.kfrac).tolist(), "kweights": np.asarray(km.weights).tolist(),
                     "fft_shape": [int(x) for x in b.fft_shape], "miller": _index_checks(b.miller),
                     "miller_rho": _index_checks(b.density_miller)}
    return out


def run_delta_q(ad):
    """The reference's Delta Q observable (observables/constraint.py: a Gaussian weight of width
    0.8 Bohr on atom 0, Delta Q = (Omega / N) sum w rho) on the fixture cell, and its derivative
    with respect to the atomic positions as central differences over full SCF runs at a fixed
    weight (Richardson over H_FD) -- the quantity the reference's implicit_grad returns."""
    from addft.geometry.cell import Cell, positions
    from addft.observables.constraint import delta_q, make_gaussian_weight
    spec = SYSTEMS["si2_gamma"]
    s = _setup(ad, spec)
    lat = np.asarray(s.geo.lattice)
    center = np.asarray(positions(s.geo))[0]
    w = np.asarray(make_gaussian_weight(s.static.basis, center, 0.8, lat))

    def dq(frac):
        s2 = _setup(ad, spec, frac)
        return float(delta_q(s2.geo, s2.static, ad.scf(s2), w))

    frac0 = np.asarray(spec["frac"], dtype=float)
    inv = np.linalg.inv(lat)
    g = np.zeros_like(frac0)
    for a in range(frac0.shape[0]):
        for c in range(3):
            d = []
            for h in H_FD:
                step = np.zeros(3)
                step[c] = h
                fp, fm = frac0.copy(), frac0.copy()
                fp[a] += step @ inv
                fm[a] -= step @ inv
                d.append((dq(fp) - dq(fm)) / (2 * h))
            g[a, c] = (4 * d[1] - d[0]) / 3
    return {"center": center.tolist(), "sigma": 0.8, "delta_q": dq(frac0), "dR_fd": g.tolist(),
            "weight_sum": float(np.sum(w))}


def run_physics(ad):
    """Reference building blocks on the Si8 differentiation cell and seeded inputs: Ewald
    energy (physics/ewald.py) with its position and strain derivatives as central differences
    (h = 1e-4, no SCF involved), the local potential on the density grid (physics/local.py),
    the Hartree potential and energy of a seeded density (physics/hartree.py), and occupations
    of seeded eigenvalues at sigma = 0.05 and 0 (physics/occupation.py)."""
    from addft.geometry.cell import Cell, strained
    from addft.physics.ewald import ewald_energy
    from addft.physics.hartree import hartree_energy, hartree_potential_r
    from addft.physics.local import local_potential_r
    from addft.physics.occupation import occupations
    spec = SI8_SYSTEMS["si8_ecut10"]
    s = _setup(ad, spec)
    geo, st = s.geo, s.static
    zval = float(np.asarray(st.psp.zval)[0])
    charges = np.full(np.asarray(geo.frac).shape[0], zval)
    lat = np.asarray(geo.lattice)
    frac0 = np.asarray(geo.frac)
    e0 = float(ewald_energy(geo, charges))
    h = 1e-4
    inv = np.linalg.inv(lat)
    dR = np.zeros_like(frac0)
    for a in range(frac0.shape[0]):
        for c in range(3):
            step = np.zeros(3)
            step[c] = h
            fp, fm = frac0.copy(), frac0.copy()
            fp[a] += step @ inv
            fm[a] -= step @ inv
            dR[a, c] = (float(ewald_energy(Cell(lattice=lat, frac=fp), charges))
                        - float(ewald_energy(Cell(lattice=lat, frac=fm), charges))) / (2 * h)
    deps = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            eps = np.zeros((3, 3))
            eps[i, j] = h
            deps[i, j] = (float(ewald_energy(strained(geo, eps), charges))
                          - float(ewald_energy(strained(geo, -eps), charges))) / (2 * h)
    vloc = np.asarray(local_potential_r(st.psp, st.spec_idx, st.basis, geo))
    rng = np.random.default_rng(5)
    rho = rng.uniform(0.0, 0.1, vloc.size)
    vh = np.asarray(hartree_potential_r(st.basis, lat, rho))
    eh = float(hartree_energy(st.basis, lat, rho))
    eig = np.sort(rng.normal(0.0, 0.3, (3, 12)), axis=1)
    wk = np.array([0.25, 0.25, 0.5])
    occ_s, mu_s = occupations(eig, wk, 14.0, 0.05)
    occ_0, _ = occupations(eig, wk, 14.0, 0.0)
    return {"ewald": e0, "ewald_dR_fd": dR.tolist(), "ewald_deps_fd": deps.tolist(), "fd_h": h,
            "vloc_r": rho_checks(vloc), "rho_seed": 5, "vh_r": rho_checks(vh), "e_hartree": eh,
            "eig": eig.tolist(), "kweights": wk.tolist(), "nelec": 14.0,
            "occ_sigma005": np.asarray(occ_s).tolist(), "mu_sigma005": float(mu_s),
            "occ_sigma0": np.asarray(occ_0).tolist()}


ABACUS_CASES = {"abacus_direct": dict(cart=False), "abacus_cartesian": dict(cart=True),
                "abacus_gamma": dict(cart=False, kpt="K_POINTS\n0\nGamma\n1 1 1 0 0 0\n")}


def run_abacus(ad):
    """The reference's ABACUS adapter (adapters/abacus/io.py setup_from_case) on the case
    directories tests/test_abacus_case.py writes: the System it builds."""
    import tempfile
    sys.path.insert(0, str(REFERENCE_SRC.parent))       # the reference's adapters/ package
    sys.path.insert(0, str(HERE.parent))
    sys.path.insert(0, str(HERE.parents[1] / "ad-dft_gb300"))   # the test module imports this package
    from test_abacus_case import _case
    out = {}
    for name, kw in ABACUS_CASES.items():
        d = _case(Path(tempfile.mkdtemp()), **kw)
        sysm = ad.setup_from_case(str(d))
        st = sysm.static
        out[name] = {"case": kw, "lattice": np.asarray(sysm.geo.lattice).tolist(),
                     "frac": np.asarray(sysm.geo.frac).tolist(), "ecut": float(st.basis.ecut),
                     "nband": int(st.nband), "sigma": float(st.sigma), "nelec": float(st.nelec),
                     "kpts": np.asarray(st.kpts).tolist(), "kweights": np.asarray(st.kweights).tolist(),
                     "nG": int(np.asarray(st.basis.miller).shape[0]),
                     "fft_shape": [int(x) for x in st.basis.fft_shape]}
    return out


def main():
    ad = _reference()
    out = HERE / "ref_fixtures.json"
    if "--system" in sys.argv and out.exists():
        name = sys.argv[sys.argv.index("--system") + 1]
        fixtures = json.loads(out.read_text())
        fixtures[name] = run_system(ad, name, SYSTEMS[name])
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--dq-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        fixtures["delta_q"] = run_delta_q(ad)
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--physics-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        fixtures["physics"] = run_physics(ad)
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--basis-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        fixtures["basis"] = run_basis(ad)
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--upf-reader-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        fixtures["upf_reader"] = run_upf(ad)
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--abacus-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        fixtures["abacus"] = run_abacus(ad)
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--si8-only" in sys.argv and out.exists():
        ad = _reference(pointwise_xc=True)
        fixtures = json.loads(out.read_text())
        for name, spec in SI8_SYSTEMS.items():
            fixtures[name] = run_system(ad, name, spec)
            fixtures[name]["xc_potential"] = "pointwise complex step of lda_energy_density"
            print(name, fixtures[name]["free_energy"], f"{fixtures[name]['seconds']:.1f} s", flush=True)
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--upf-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        for name, spec in UPF_SYSTEMS.items():
            fixtures[name] = run_system(ad, name, spec)
            print(name, fixtures[name]["free_energy"], f"{fixtures[name]['seconds']:.1f} s", flush=True)
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--stress-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        fixtures["si2_gamma"]["stress_fd"] = stress_fd(ad, _setup(ad, SYSTEMS["si2_gamma"])).tolist()
        out.write_text(json.dumps(fixtures, indent=1))
        return
    if "--micro-only" in sys.argv and out.exists():
        fixtures = json.loads(out.read_text())
        fixtures["microbench"] = {str(n): run_micro(ad, n) for n in MICRO_BOXES}
        out.write_text(json.dumps(fixtures, indent=1))
        return
    fixtures = {"generator": "tests/golden/make_reference_fixtures.py (reference code on NumPy via refshim)"}
    for name, spec in {**SYSTEMS, **UPF_SYSTEMS}.items():
        fixtures[name] = run_system(ad, name, spec)
        print(name, fixtures[name]["free_energy"], f"{fixtures[name]['seconds']:.1f} s", flush=True)
    fixtures["microbench"] = {str(n): run_micro(ad, n) for n in MICRO_BOXES}
    fixtures["abacus"] = run_abacus(ad)
    fixtures["upf_reader"] = run_upf(ad)
    fixtures["basis"] = run_basis(ad)
    fixtures["physics"] = run_physics(ad)
    fixtures["delta_q"] = run_delta_q(ad)
    ad = _reference(pointwise_xc=True)
    for name, spec in SI8_SYSTEMS.items():
        fixtures[name] = run_system(ad, name, spec)
        fixtures[name]["xc_potential"] = "pointwise complex step of lda_energy_density"
        print(name, fixtures[name]["free_energy"], f"{fixtures[name]['seconds']:.1f} s", flush=True)
    (HERE / "ref_fixtures.json").write_text(json.dumps(fixtures, indent=1))


if __name__ == "__main__":
    main()
