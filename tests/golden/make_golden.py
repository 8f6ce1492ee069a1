"""Writes tests/golden/cfg1_si2_fixture.json from the NumPy oracle.

The oracle is pinned to the reference's recorded fixture values by
tests/test_oracle_pins.py; this file freezes its outputs on the reference's
own fixture system (tests/conftest.py:26-34 of ad-dft: 6 Bohr cubic cell,
frac (0,0,0)/(0.53,0.47,0.49), ecut 2 Ha, nband 2, density_factor 4,
sigma 0.05, synthetic pseudopotential) so GPU runs compare against fixed
numbers.  Run:  python tests/golden/make_golden.py
"""

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import pw  # noqa: E402


def main():
    s = pw.setup(np.eye(3) * 6.0, [[0, 0, 0], [0.53, 0.47, 0.49]], ecut=2.0, nband=2,
                 density_factor=4.0, sigma=0.05)
    st = pw.solve_scf(s)
    dR, deps = pw.envelope_gradients(s, st)
    out = {
        "system": "reference fixture: 6 Bohr cubic, frac (0,0,0)/(0.53,0.47,0.49), ecut 2, nband 2, "
                  "density_factor 4, sigma 0.05, synthetic psp",
        "nG": s.static.basis.nG, "fft_shape": list(s.static.basis.fft_shape),
        "scf_iterations": st.n_iter, "residual": st.residual,
        "free_energy": pw.mermin_free_energy(s, st),
        "energy_terms": pw.energy_terms(s, st),
        "eig": st.eig.tolist(), "occ": st.occ.tolist(), "mu": st.mu,
        "forces": (-dR).tolist(),
        "stress": pw.stress_from_deps(pw.volume(s.lattice), deps).tolist(),
        "recorded_reference_energy_pre_vloc_fix": -2.57875,
    }
    path = Path(__file__).resolve().parent / "cfg1_si2_fixture.json"
    path.write_text(json.dumps(out, indent=1, default=float) + "\n")
    print(path)


if __name__ == "__main__":
    main()
