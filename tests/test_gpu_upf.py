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


def twin(ecut=4.0, nband=6, kmesh=None):
    s = ad.setup(LATTICE, FRAC_DISTORTED, psp=ad.from_upf(V2), ecut=ecut, nband=nband,
                 kmesh=ad.monkhorst_pack(kmesh) if kmesh else None)
    o = pw.setup(LATTICE, FRAC_DISTORTED, psp=pw.from_upf(V2), ecut=ecut, nband=nband,
                 kmesh=pw.monkhorst_pack(kmesh) if kmesh else None)
    return s, o


@pytest.mark.parametrize("kmesh", [None, (2, 2, 2)])
def test_upf_tables_on_gpu_match_oracle(kmesh):
    s, o = twin(kmesh=kmesh)
    cache = build_geometry_cache(s.geo, s.static)
    oc = pw.build_geometry_cache(o.static, o.lattice, o.frac)
    proj = cache.proj.cpu().numpy()
    assert np.max(np.abs(proj - oc.proj)) < 1e-9 * np.max(np.abs(oc.proj))
    v = cache.v_loc_r.cpu().numpy()
    assert np.max(np.abs(v - oc.v_loc_r)) < 1e-9 * np.max(np.abs(oc.v_loc_r))


def test_upf_scf_energy_forces_stress_match_oracle():
    s, o = twin()
    st = ad.scf(s)
    ost = pw.solve_scf(o)
    e = obs.mermin_free_energy(s.geo, s.static, st)
    assert abs(e - pw.mermin_free_energy(o, ost)) < 1e-8
    assert np.max(np.abs(st.eig.cpu().numpy() - ost.eig)) < 1e-8
    dR, deps = obs.envelope_gradients(s.geo, s.static, st)
    odR, odeps = pw.envelope_gradients(o, ost)
    assert np.max(np.abs(dR - odR)) < 1e-7
    assert np.max(np.abs(deps - odeps)) < 1e-7
