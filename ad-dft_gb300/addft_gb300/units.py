"""Units (src/addft/runtime/units.py:12-33): Hartree / Bohr inside, Ry bridge at I/O only."""

HA_TO_EV = 27.211386245988
RY_TO_HA = 0.5
BOHR_TO_ANG = 0.529177210903
ANG_TO_BOHR = 1.0 / BOHR_TO_ANG
HA_TO_KBAR = 2.942105e5


def ry_to_ha(x):
    return x * RY_TO_HA


def ha_to_ry(x):
    return x / RY_TO_HA


def ha_to_ev(x):
    return x * HA_TO_EV


def stress_ha_bohr3_to_kbar(s):
    return s * HA_TO_KBAR
