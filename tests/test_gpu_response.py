"""GPU linear response, fixed-point adjoint and Delta Q gradient against the oracle.

The oracle builds the response from the full dense eigensystem; the GPU path is
matrix-free (window sum + Sternheimer CG with FP64 H psi).  Tolerances: response
1e-9 relative, adjoint gradients 1e-7 absolute (the oracle's map derivative is a
central difference with h = 1e-5).
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import FRAC_DISTORTED, LATTICE, gpu_available

pytestmark = pytest.mark.gpu
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import torch  # noqa: E402

import addft_gb300 as ad  # noqa: E402
from addft_gb300 import observables as obs  # noqa: E402
from addft_gb300.response import Response  # noqa: E402
from oracle import pw  # noqa: E402


def twin(nband=7, kmesh=None, ecut=2.0):
    s = ad.setup(LATTICE, FRAC_DISTORTED, ecut=ecut, nband=nband,
                 kmesh=ad.monkhorst_pack(kmesh) if kmesh else None)
    o = pw.setup(LATTICE, FRAC_DISTORTED, ecut=ecut, nband=nband,
                 kmesh=pw.monkhorst_pack(kmesh) if kmesh else None)
    return s, o


@pytest.mark.parametrize("kmesh,nband", [(None, 7), ((2, 2, 2), 8)])
def test_response_matches_dense_oracle(kmesh, nband):
    # band windows whose top lies in a gap at every k (>= 1.5e-2 Ha): the map is smooth there
    s, o = twin(kmesh=kmesh, nband=nband)
    st = ad.scf(s)
    ost = pw.solve_scf(o)
    apply_o, _ = pw.make_response(o, ost)
    resp = Response(s.geo, s.static, st)
    rng = np.random.default_rng(3)
    for _ in range(2):
        dn = rng.normal(size=o.static.basis.nfft) * 1e-3
        got = resp.apply(torch.as_tensor(dn, device="cuda")).cpu().numpy()
        want = apply_o(dn)
        assert np.max(np.abs(got - want)) < 1e-9 * np.max(np.abs(want))


def test_transposed_response_is_kernel_times_chi0():
    s, _ = twin()
    st = ad.scf(s)
    resp = Response(s.geo, s.static, st)
    rng = np.random.default_rng(4)
    x = torch.as_tensor(rng.normal(size=s.static.basis.nfft), device="cuda")
    y = torch.as_tensor(rng.normal(size=s.static.basis.nfft), device="cuda")
    a = float(torch.dot(y, resp.apply(x)))
    b = float(torch.dot(resp.apply_t(y), x))
    assert abs(a - b) < 1e-10 * max(abs(a), 1.0)


def test_delta_q_gradient_matches_oracle_adjoint():
    s, o = twin()
    st = ad.scf(s)
    ost = pw.solve_scf(o)
    center = pw.positions(o.lattice, o.frac)[0]
    w = pw.make_gaussian_weight(o.static.basis, center, 0.8, o.lattice)
    assert np.allclose(obs.make_gaussian_weight(s.static.basis, center, 0.8, LATTICE), w)
    assert abs(obs.delta_q(s.geo, s.static, st, w) - pw.delta_q(o, ost, w)) < 1e-11
    grad, diag = obs.delta_q_grad(s.geo, s.static, st, w)
    dR, deps, _ = pw.implicit_grad_delta_q(o, ost, w)
    assert diag["adjoint_residual"] < 1e-9
    assert np.max(np.abs(diag["dR"] - dR)) < 1e-7
    assert np.max(np.abs(diag["deps"] - deps)) < 1e-7
    assert np.allclose(grad.frac, dR @ LATTICE.T, atol=1e-6)


@pytest.mark.slow
def test_delta_q_gradient_si8_matches_full_scf_differences():
    """The differentiation workload: Si8 conventional cell (a = 10.26, seeded 0.05 Bohr
    displacements), ecut 10 Ha, Gamma, 20 bands (nG 1647, above the dense cutoff, so
    the FP64 Davidson buffer and the Sternheimer CG run): the matrix-free adjoint
    against central differences of Delta Q over full SCF runs (h = 1e-3 Bohr)."""
    a = 10.26
    base = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                     [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
    frac = base + np.random.default_rng(8).normal(0, 0.05, base.shape) / a
    lat = np.eye(3) * a
    s = ad.setup(lat, frac, ecut=10.0, nband=20)
    st = ad.scf(s)
    center = frac[0] @ lat
    w = obs.make_gaussian_weight(s.static.basis, center, 1.2, lat)
    grad, diag = obs.delta_q_grad(s.geo, s.static, st, w)
    assert diag["adjoint_residual"] < 1e-8
    print("Si8 Delta Q adjoint:", {k: v for k, v in diag.items() if k not in ("dR", "deps")})
    h = 1e-3
    for i, ax in ((0, 0), (3, 1)):
        qs = []
        for sgn in (1, -1):
            pos = frac @ lat
            pos[i, ax] += sgn * h
            s2 = ad.setup(lat, pos @ np.linalg.inv(lat), ecut=10.0, nband=20)
            qs.append(obs.delta_q(s2.geo, s2.static, ad.scf(s2), w))
        fd = (qs[0] - qs[1]) / (2 * h)
        print("dQ/dR", i, ax, "adjoint", diag["dR"][i, ax], "central difference", fd)
        assert abs(fd - diag["dR"][i, ax]) < 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("adjoint_mode", ["matrix_free", "dense"])
def test_make_energy_adjoint_mode_matches_oracle(adjoint_mode):
    """make_energy(static, mode="adjoint") (reference api.py:114-116): value_and_grad through
    the fixed-point adjoint against the oracle's dense adjoint of the same quantity
    (pw.implicit_grad_energy, itself pinned by full-SCF central differences), 1e-7."""
    s, o = twin(nband=2)
    ost = pw.solve_scf(o)
    dR, deps = pw.implicit_grad_energy(o, ost)
    f = ad.make_energy(s.static, mode="adjoint", adjoint_mode=adjoint_mode)
    e, g = f.value_and_grad(s.geo)
    assert abs(e - pw.mermin_free_energy(o, ost)) < 2e-8
    assert np.max(np.abs(g.frac - dR @ LATTICE.T)) < 1e-7
    assert np.max(np.abs(g.lattice - np.linalg.inv(LATTICE).T @ deps)) < 1e-7
    # the envelope mode of the same function gives the physical forces, which differ
    fe = ad.make_energy(s.static, mode="envelope")
    _, ge = fe.value_and_grad(s.geo)
    edR, _ = pw.envelope_gradients(o, ost)
    assert np.max(np.abs(ge.frac - edR @ LATTICE.T)) < 1e-7
    with pytest.raises(ValueError):
        ad.make_energy(s.static, mode="adjoint", adjoint_mode="bogus")


def test_delta_q_adjoint_matches_reference_code_differences():
    """The GPU matrix-free adjoint derivative of Delta Q with respect to the atomic positions
    against central differences of the reference's own Delta Q over full SCF runs
    (tests/golden/make_reference_fixtures.py): 1e-7 absolute."""
    import json
    from pathlib import Path
    c = json.loads((Path(__file__).resolve().parent / "golden" / "ref_fixtures.json").read_text())["delta_q"]
    s, o = twin(nband=2)   # the fixture cell as the reference ran it
    st = ad.scf(s)
    w = obs.make_gaussian_weight(s.static.basis, np.asarray(c["center"]), c["sigma"], LATTICE)
    assert abs(obs.delta_q(s.geo, s.static, st, w) - c["delta_q"]) < 1e-11
    _, diag = obs.delta_q_grad(s.geo, s.static, st, w)
    assert np.max(np.abs(diag["dR"] - np.asarray(c["dR_fd"]))) < 1e-7
