"""Forces and stress of the differentiation workload against central differences.

Si8 conventional diamond cell (a = 10.26 Bohr, seeded 0.05 Bohr displacements), ecut
10 Ha, Gamma only, 20 bands: the GPU envelope gradients (the VJP kernels behind
``energy_and_forces`` and ``stress``) against central differences of the Mermin free
energy over full SCF runs with h = 1e-3 (Bohr for displacements, dimensionless for
strain; strain also at h/2, with Richardson extrapolation).  The basis is held fixed
under strain (``make_energy(static)``), which is the derivative the analytic stress is.
Bars: 1e-6 for the FP64 path (the reference's gradient-vs-FD bar), 1e-5 for FP32 H psi
with FP64 refinement.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import addft_gb300 as ad  # noqa: E402
from addft_gb300 import observables as obs  # noqa: E402
from addft_gb300.geometry import displacement, strained  # noqa: E402

H = 1e-3


@pytest.fixture(scope="module")
def si8():
    a = 10.26
    base = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                     [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
    frac = base + np.random.default_rng(8).normal(0, 0.05, base.shape) / a
    s = ad.setup(np.eye(3) * a, frac, ecut=10.0, nband=20)
    st = ad.scf(s)
    dR, deps = obs.envelope_gradients(s.geo, s.static, st)
    return s, st, dR, deps, ad.make_energy(s.static)


def _central(f, plus, minus):
    return (f(plus) - f(minus)) / (2 * H)


def test_si8_forces_match_central_differences(si8):
    s, st, dR, _, f = si8
    e, forces = ad.energy_and_forces(s)
    assert np.allclose(forces, -dR, atol=1e-10)
    assert np.max(np.abs(forces.sum(axis=0))) < 1e-6
    for i, ax in ((0, 0), (3, 1), (6, 2)):
        d = np.zeros((8, 3))
        d[i, ax] = H
        fd = _central(f, displacement(s.geo, d), displacement(s.geo, -d))
        print(f"dF/dR[{i},{ax}] analytic {dR[i, ax]:+.10f} central difference {fd:+.10f}")
        assert abs(fd - dR[i, ax]) < 1e-6


def test_si8_stress_matches_central_differences(si8):
    """Strain derivatives: the central difference at h carries an h^2 term of a few
    1e-6 here (the energy's third strain derivative is tens of Ha), so the check is
    that the difference at h/2 is closer by about 4x and that the Richardson
    extrapolation (4 D(h/2) - D(h)) / 3 matches to 1e-6."""
    s, st, _, deps, f = si8
    sig = ad.stress(s, st)
    omega = abs(np.linalg.det(s.geo.lattice))
    assert np.allclose(sig, obs.stress_from_deps(omega, deps), atol=1e-14)
    for i, j in ((0, 0), (1, 1), (0, 1), (1, 2)):
        unit = np.zeros((3, 3))
        unit[i, j] += 0.5
        unit[j, i] += 0.5
        d1 = _central(f, strained(s.geo, H * unit), strained(s.geo, -H * unit))
        d2 = _central(f, strained(s.geo, 0.5 * H * unit), strained(s.geo, -0.5 * H * unit)) * 2.0
        rich = (4 * d2 - d1) / 3
        an = 0.5 * (deps[i, j] + deps[j, i])
        print(f"dF/deps[{i},{j}] analytic {an:+.10f} central h {d1:+.10f} h/2 {d2:+.10f} Richardson {rich:+.10f}")
        scale = max(1.0, abs(an))
        assert abs(d1 - an) < 2e-5 * scale
        assert abs(rich - an) < 1e-6 * scale
        assert abs(d2 - an) < 0.5 * abs(d1 - an) + 1e-7 * scale


def test_si8_fp32_refined_gradients_match_central_differences(si8):
    s, st, dR, deps, f = si8
    e32, f32 = ad.energy_and_forces(s, precision="fp32")
    assert abs(e32 - ad.energy(s, st)) / 8 < 1e-6
    assert np.max(np.abs(f32 + dR)) < 1e-5
    sig32 = ad.stress(s, precision="fp32")
    omega = abs(np.linalg.det(s.geo.lattice))
    assert np.max(np.abs(sig32 - obs.stress_from_deps(omega, deps))) < 1e-5 / omega
    # one displacement through the FP32 path end to end
    f32e = ad.make_energy(s.static, precision="fp32")
    d = np.zeros((8, 3))
    d[5, 0] = H
    fd = _central(f32e, displacement(s.geo, d), displacement(s.geo, -d))
    assert abs(fd - dR[5, 0]) < 1e-5
