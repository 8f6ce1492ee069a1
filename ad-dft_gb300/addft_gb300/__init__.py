"""addft_gb300: the ad-dft plane-wave hot path on GB300 (sm_103a), same API.

    import addft_gb300 as ad
    s = ad.setup(lattice=[[6., 0, 0], [0, 6., 0], [0, 0, 6.]],
                 frac=[[0, 0, 0], [0.53, 0.47, 0.49]], ecut=2.0, nband=2)
    E, F = ad.energy_and_forces(s)
    sigma = ad.stress(s)
    terms = ad.energy_decomposition(s)

Every heavy step runs in libaddft_gb300.so (hand-written CUDA for sm_103a,
reached through a plain C ABI); there is no CPU fallback.
"""

from . import units  # noqa: F401
from .api import (System, energy, energy_and_forces, energy_decomposition, energy_explicit,  # noqa: F401
                  make_energy, scf, setup, setup_from_case, stress)
from .geometry import Cell, gamma, monkhorst_pack, strained, volume  # noqa: F401
from .psp import Pseudo, from_upf, synthetic  # noqa: F401

__all__ = [
    "System", "setup", "setup_from_case", "scf", "energy", "energy_explicit", "energy_and_forces", "stress",
    "energy_decomposition", "make_energy", "Cell", "strained", "volume", "gamma", "monkhorst_pack", "Pseudo",
    "synthetic", "from_upf", "units",
]
