"""UPF pseudopotential on the GPU path against the oracle (exact quadratures).

The kernels read the radial functions from the cubic Hermite table, so the
parity bar is the table's accuracy (~1e-11 relative) rather than FP64
rounding: 1e-9 on tables, 1e-8 Ha on energies, 1e-7 on forces and strain
derivatives.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from conftest import FRAC_DISTORTED, LATTICE, gpu_available

pytestmark = pytest.mark.gpu
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import torch  # noqa: E402

import addft_gb300 as ad  # noqa: E402
from addft_gb300 import observables as obs  # noqa: E402
from addft_gb300.system import build_geometry_cache  # noqa: E402
from oracle import pw  # noqa: E402

V2 = Path(__file__).resolve().parent / "golden" / "si_test_v2.upf"
D2 = Path(__file__).resolve().parent / "golden" / "si_test_d_v2.upf"   # adds an l = 2 projector


def twin(ecut=4.0, nband=6, kmesh=None, path=V2):
    s = ad.setup(LATTICE, FRAC_DISTORTED, psp=ad.from_upf(path), ecut=ecut, nband=nband,
                 kmesh=ad.monkhorst_pack(kmesh) if kmesh else None)
    o = pw.setup(LATTICE, FRAC_DISTORTED, psp=pw.from_upf(path), ecut=ecut, nband=nband,
                 kmesh=pw.monkhorst_pack(kmesh) if kmesh else None)
    return s, o


@pytest.mark.parametrize("kmesh,path", [(None, V2), ((2, 2, 2), V2), ((2, 2, 2), D2)])
def test_upf_tables_on_gpu_match_oracle(kmesh, path):
    s, o = twin(kmesh=kmesh, path=path)
    cache = build_geometry_cache(s.geo, s.static)
    oc = pw.build_geometry_cache(o.static, o.lattice, o.frac)
    proj = cache.proj.cpu().numpy()
    assert np.max(np.abs(proj - oc.proj)) < 1e-9 * np.max(np.abs(oc.proj))
    v = cache.v_loc_r.cpu().numpy()
    assert np.max(np.abs(v - oc.v_loc_r)) < 1e-9 * np.max(np.abs(oc.v_loc_r))


@pytest.mark.parametrize("path", [V2, D2])
def test_upf_scf_energy_forces_stress_match_oracle(path):
    """s + p channels, and s + p + d channels (the d projector through the l = 2 real Y_lm
    of ylm.py:18-25 and its gradient in the force and stress kernels)."""
    s, o = twin(path=path)
    st = ad.scf(s)
    ost = pw.solve_scf(o)
    e = obs.mermin_free_energy(s.geo, s.static, st)
    assert abs(e - pw.mermin_free_energy(o, ost)) < 1e-8
    assert np.max(np.abs(st.eig.cpu().numpy() - ost.eig)) < 1e-8
    dR, deps = obs.envelope_gradients(s.geo, s.static, st)
    odR, odeps = pw.envelope_gradients(o, ost)
    assert np.max(np.abs(dR - odR)) < 1e-7
    assert np.max(np.abs(deps - odeps)) < 1e-7


def test_synthetic_d_projector_scf_forces_stress_match_oracle():
    """The reference's synthetic() with three projectors gives l = 0, 1, 2 (psp.py:141-164):
    projector tables, SCF energy, forces and stress against the oracle."""
    kw = dict(proj_w=(1.0, 0.6, 0.5), proj_b=(0.9, 1.4, 1.1), dion_diag=(-2.0, -0.7, 0.6))
    s = ad.setup(LATTICE, FRAC_DISTORTED, psp=ad.synthetic(**kw), ecut=3.0, nband=6)
    o = pw.setup(LATTICE, FRAC_DISTORTED, psp=pw.synthetic(**kw), ecut=3.0, nband=6)
    assert s.static.psp.proj_l == (0, 1, 2) and s.static.psp.nh == 9
    cache = build_geometry_cache(s.geo, s.static)
    oc = pw.build_geometry_cache(o.static, o.lattice, o.frac)
    assert np.max(np.abs(cache.proj.cpu().numpy() - oc.proj)) < 1e-13
    st = ad.scf(s)
    ost = pw.solve_scf(o)
    assert abs(obs.mermin_free_energy(s.geo, s.static, st) - pw.mermin_free_energy(o, ost)) < 1e-8
    dR, deps = obs.envelope_gradients(s.geo, s.static, st)
    odR, odeps = pw.envelope_gradients(o, ost)
    assert np.max(np.abs(dR - odR)) < 1e-7
    assert np.max(np.abs(deps - odeps)) < 1e-7
