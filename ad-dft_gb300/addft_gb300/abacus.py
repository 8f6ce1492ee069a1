"""ABACUS case directories (INPUT / KPT / STRU + UPF) -> System
(adapters/abacus/io.py:1-236).

Rules, as in the reference adapter: units are converted once, here (ABACUS's
Ry energies -> Ha); every INPUT key must be mapped or is an error, and the
keys the path does not support are errors too (a silently ignored parameter
gives a run that looks fine and is wrong); atoms are bound to their
ATOMIC_SPECIES block; Cartesian positions are in units of LATTICE_CONSTANT.
One species per case, as the GPU path.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np

RY_TO_HA = 0.5


def _flag(v) -> bool:
    return int(v) != 0


#: INPUT key -> (field, conversion)   (io.py:21-44)
PARAM_MAP = {
    "ecutwfc": ("basis.ecut_ha", lambda v: float(v) * RY_TO_HA),
    "nbands": ("nband", int),
    "pseudo_dir": ("pseudo_dir", str),
    "cal_force": ("scf.cal_force", _flag),
    "cal_stress": ("scf.cal_stress", _flag),
    "out_element_info": ("scf.out_element_info", _flag),
    "ntype": ("cell.ntype", int),
    "suffix": ("io.suffix", str),
    "ks_solver": ("solver.ks_solver", str),
    "scf_thr": ("scf.threshold", float),
    "scf_nmax": ("scf.max_iter", int),
    "smearing_method": ("occupation.method", str),
    "smearing_sigma": ("occupation.sigma_ha", lambda v: float(v) * RY_TO_HA),
    "mixing_type": ("scf.mixer", str),
    "mixing_beta": ("scf.beta", float),
    "nspin": ("spin.nspin", int),
    "symmetry": ("symmetry.enabled", _flag),
    "dft_functional": ("xc.name", str),
    "basis_type": ("basis.type", str),
    "device": ("runtime.device", str),
    "calculation": ("task.type", str),
}

#: keys the plane-wave path does not provide (io.py:47-52)
UNSUPPORTED = {
    "dft_plus_u": "DFT+U is not provided",
    "orbital_dir": "numerical atomic orbital bases are not provided",
    "vdw_method": "vdW corrections are not provided",
}


class UnmappedParameterError(KeyError):
    pass


def _lines(path):
    for raw in Path(path).read_text(encoding="utf-8").splitlines():
        line = raw.split("#")[0].strip()
        if line:
            yield line


def parse_input(path) -> dict:
    """INPUT: `key value` lines after an optional INPUT_PARAMETERS header (io.py:64-86)."""
    out = {}
    for line in _lines(path):
        parts = line.split()
        key = parts[0].lower()
        if key == "input_parameters":
            continue
        if len(parts) < 2:
            raise UnmappedParameterError(f"INPUT line without a value: {line!r}")
        if key in UNSUPPORTED:
            raise UnmappedParameterError(f"{key}: {UNSUPPORTED[key]}")
        if key not in PARAM_MAP:
            raise UnmappedParameterError(f"INPUT parameter {key!r} has no mapping; add it to PARAM_MAP "
                                         "rather than ignoring it")
        field, conv = PARAM_MAP[key]
        out[field] = conv(parts[1])
    if out.get("spin.nspin", 1) != 1:
        raise UnmappedParameterError("nspin != 1: spin-polarised runs are not provided")
    return out


def parse_kpt(path) -> dict:
    """KPT: {"mode": "gamma"} when the file names Gamma anywhere (the reference's reading,
    io.py:89-109), else a Monkhorst-Pack mesh with shifts given in half steps."""
    tokens = [t for line in _lines(path) for t in line.split()]
    if not tokens:
        raise ValueError("empty KPT file")
    if "Gamma" in tokens:
        return {"mode": "gamma"}
    i = tokens.index("Monkhorst-Pack") if "Monkhorst-Pack" in tokens else 0
    nums = [int(float(x)) for x in tokens[i + 1:i + 7]]
    return {"mode": "mp", "mesh": tuple(nums[:3]), "shift": tuple(x / 2.0 for x in nums[3:6])}


def parse_stru(path) -> dict:
    """STRU: lattice (Bohr) = LATTICE_VECTORS x LATTICE_CONSTANT; positions Direct or
    Cartesian (in LATTICE_CONSTANT units); atoms bound to their species (io.py:112-206)."""
    text = [ln.split("#")[0].rstrip() for ln in Path(path).read_text(encoding="utf-8").splitlines()]
    lat0, vecs, labels, pseudo_files = 1.0, [], [], []
    species, coords, magmoms = [], [], []
    mode, i, n = None, 0, len(text)
    while i < n:
        line = text[i].strip()
        if not line:
            i += 1
            continue
        if line.startswith("ATOMIC_SPECIES"):
            i += 1
            while i < n:
                s = text[i].strip()
                if not s:
                    i += 1
                    continue
                if s.startswith(("LATTICE_", "ATOMIC_", "NUMERICAL_")):
                    break
                parts = s.split()
                if len(parts) >= 3:
                    labels.append(parts[0])
                    pseudo_files.append(parts[2])
                i += 1
            continue
        if line.startswith("LATTICE_CONSTANT"):
            parts = line.split()
            if len(parts) >= 2:
                lat0, i = float(parts[1]), i + 1
            else:
                lat0, i = float(text[i + 1].strip()), i + 2
            continue
        if line.startswith("LATTICE_VECTORS"):
            vecs = [[float(x) for x in text[i + 1 + j].split()[:3]] for j in range(3)]
            i += 4
            continue
        if line.startswith("ATOMIC_POSITIONS"):
            parts = line.split()
            i += 1
            if len(parts) >= 2:
                mode = parts[1]
            else:
                while i < n and not text[i].strip():
                    i += 1
                mode, i = text[i].strip().split()[0], i + 1
            if mode not in ("Direct", "Cartesian"):
                raise NotImplementedError(f"coordinate mode {mode!r} is not provided (Direct, Cartesian)")
            break
        i += 1
    while i < n:
        s = text[i].strip()
        if not s:
            i += 1
            continue
        if s.startswith(("LATTICE_", "ATOMIC_")):
            break
        label = s.split()[0]
        if label not in labels:
            raise ValueError(f"ATOMIC_POSITIONS species {label!r} is not in ATOMIC_SPECIES")
        mag = float(text[i + 1].split()[0])
        count = int(float(text[i + 2].split()[0]))
        i += 3
        for _ in range(count):
            coords.append([float(x) for x in text[i].split()[:3]])
            magmoms.append(mag)
            species.append(label)
            i += 1
    if mode is None:
        raise ValueError("STRU without ATOMIC_POSITIONS")
    lat = np.asarray(vecs, dtype=np.float64) * lat0
    c = np.asarray(coords, dtype=np.float64)
    frac = c if mode == "Direct" else (c * lat0) @ np.linalg.inv(lat)
    return dict(lattice=lat, frac=frac, species=species, magmoms=np.asarray(magmoms), labels=labels,
                pseudo_files=pseudo_files)


def setup_from_case(case_dir):
    """System from an ABACUS case directory: INPUT, KPT, STRU and the UPF named in STRU
    under pseudo_dir (io.py:209-230).  Smearing width from smearing_sigma (Ry),
    0 for smearing_method fixed, otherwise 0.05 Ha."""
    from .api import setup
    from .geometry import gamma, monkhorst_pack
    from .psp import from_upf

    case = Path(case_dir)
    inp = parse_input(case / "INPUT")
    kpt = parse_kpt(case / "KPT")
    stru = parse_stru(case / "STRU")
    if len(set(stru["species"])) != 1:
        raise NotImplementedError("one species per case (multi-species cells are rejected)")
    label = stru["species"][0]
    psp = from_upf(case / inp.get("pseudo_dir", ".") / stru["pseudo_files"][stru["labels"].index(label)])
    km = gamma() if kpt["mode"] == "gamma" else monkhorst_pack(kpt["mesh"], kpt["shift"])
    sigma = 0.0 if inp.get("occupation.method") == "fixed" else inp.get("occupation.sigma_ha", 0.05)
    if "basis.ecut_ha" not in inp:
        raise UnmappedParameterError("INPUT has no ecutwfc")
    return setup(lattice=stru["lattice"], frac=stru["frac"], psp=psp, ecut=inp["basis.ecut_ha"],
                 nband=inp.get("nband", 6), kmesh=km, sigma=sigma)
