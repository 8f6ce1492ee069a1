"""ABACUS case directories (INPUT, KPT, STRU and the UPF files STRU names) as
``setup()`` arguments, the entry of the reference's ABACUS adapter
(adapters/abacus/io.py; api.setup_from_case).

INPUT: every keyword has a role in ``INPUT_KEYWORDS``; a keyword without one is
an error, never silently ignored (a run that drops a parameter looks fine and is
wrong).  Roles:
  setup    converted onto an ``addft.setup`` argument (energies Ry -> Ha);
  scf      converted onto a ``solve_scf`` keyword (kept in ``AbacusCase.scf_args``);
  task     what the case asks to compute (``AbacusCase.tasks``);
  file     where the case's other files are;
  require  must have the one value this path implements (else an error);
  accept   recorded in ``AbacusCase.info``; does not change the plane-wave fixed point
           (solver choice, mixing scheme, output options, device);
  reject   a feature this path does not provide (error).
KPT: ``K_POINTS`` / count / type / ``n1 n2 n3 s1 s2 s3``.  As in the reference
adapter, a file whose type is Gamma means the Gamma point alone, and
Monkhorst-Pack shifts 0/1 are half steps.
STRU: sections split on their ABACUS keywords, each read by its own parser;
lattice in Bohr = LATTICE_VECTORS x LATTICE_CONSTANT; Cartesian positions in
units of LATTICE_CONSTANT; every atom bound to an ATOMIC_SPECIES label.
One species per case, as the GPU path.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

RY_TO_HA = 0.5


class UnmappedParameterError(KeyError):
    pass


def _ry(v: str) -> float:
    return float(v) * RY_TO_HA


def _onoff(v: str) -> bool:
    return v.strip().lower() in ("1", "true", "t", ".true.", "yes")


_LDA_NAMES = ("lda", "pz", "pz-lda", "lda_pz", "slater-pz", "sla+pz", "default")

#: ABACUS INPUT keyword -> (role, target, converter)
INPUT_KEYWORDS = {
    "ecutwfc": ("setup", "ecut", _ry),
    "nbands": ("setup", "nband", int),
    "smearing_sigma": ("setup", "sigma", _ry),
    "smearing_method": ("task", "smearing", str.lower),
    "pseudo_dir": ("file", "pseudo_dir", str),
    "stru_file": ("file", "stru_file", str),
    "kpoint_file": ("file", "kpoint_file", str),
    "scf_thr": ("scf", "tol", float),
    "scf_nmax": ("scf", "max_iter", int),
    "mixing_beta": ("scf", "beta", float),
    "calculation": ("task", "calculation", str.lower),
    "cal_force": ("task", "cal_force", _onoff),
    "cal_stress": ("task", "cal_stress", _onoff),
    "ntype": ("require", 1, int),
    "nspin": ("require", 1, int),
    "basis_type": ("require", "pw", str.lower),
    "dft_functional": ("require", _LDA_NAMES, str.lower),
    "ks_solver": ("accept", None, str),
    "mixing_type": ("accept", None, str),
    "symmetry": ("accept", None, str),
    "suffix": ("accept", None, str),
    "out_element_info": ("accept", None, str),
    "device": ("accept", None, str),
    "dft_plus_u": ("reject", "DFT+U is not provided", None),
    "orbital_dir": ("reject", "numerical atomic orbital bases are not provided", None),
    "vdw_method": ("reject", "vdW corrections are not provided", None),
    "lspinorb": ("reject", "spin-orbit coupling is not provided", None),
    "noncolin": ("reject", "non-collinear spin is not provided", None),
}


@dataclass
class AbacusInput:
    setup_args: dict = field(default_factory=dict)
    scf_args: dict = field(default_factory=dict)
    tasks: dict = field(default_factory=dict)
    files: dict = field(default_factory=dict)
    info: dict = field(default_factory=dict)


def _rows(path) -> list:
    """Token rows of a file, '#' and '//' comments and blank lines removed."""
    rows = []
    for raw in Path(path).read_text(encoding="utf-8").splitlines():
        line = raw.split("#")[0].split("//")[0].strip()
        if line:
            rows.append(line.split())
    return rows


def read_input(path) -> AbacusInput:
    """INPUT: an optional INPUT_PARAMETERS line, then `keyword value` rows."""
    out = AbacusInput()
    for row in _rows(path):
        key = row[0].lower()
        if key == "input_parameters":
            continue
        if key not in INPUT_KEYWORDS:
            raise UnmappedParameterError(f"INPUT keyword {key!r} has no role on this path; give it one in "
                                         "INPUT_KEYWORDS instead of ignoring it")
        role, target, conv = INPUT_KEYWORDS[key]
        if role == "reject":
            raise UnmappedParameterError(f"{key}: {target}")
        if len(row) < 2:
            raise UnmappedParameterError(f"INPUT keyword {key!r} has no value")
        value = conv(row[1])
        if role == "require":
            ok = value in target if isinstance(target, tuple) else value == target
            if not ok:
                raise UnmappedParameterError(f"{key} = {row[1]}: this path provides only {target}")
        elif role == "setup":
            out.setup_args[target] = value
        elif role == "scf":
            out.scf_args[target] = value
        elif role == "task":
            out.tasks[target] = value
        elif role == "file":
            out.files[target] = value
        else:
            out.info[key] = value
    return out


def read_kpt(path) -> dict:
    """KPT rows: K_POINTS, the point count (0: a generated mesh), the type, the mesh."""
    rows = [r for r in _rows(path) if r[0].upper() != "K_POINTS"]
    if not rows:
        raise ValueError("empty KPT file")
    kinds = [r[0].lower() for r in rows]
    if "gamma" in kinds:
        return {"mode": "gamma"}
    for i, k in enumerate(kinds):
        if k in ("monkhorst-pack", "mp") and i + 1 < len(rows):
            n = [int(float(x)) for x in rows[i + 1][:6]]
            n += [0] * (6 - len(n))
            return {"mode": "mp", "mesh": tuple(n[:3]), "shift": tuple(s / 2.0 for s in n[3:6])}
    raise NotImplementedError("KPT: only Gamma and Monkhorst-Pack meshes are provided")


# ---------------------------------------------------------------------------
# STRU
# ---------------------------------------------------------------------------
STRU_SECTIONS = ("ATOMIC_SPECIES", "NUMERICAL_ORBITAL", "LATTICE_CONSTANT", "LATTICE_VECTORS",
                 "LATTICE_PARAMETERS", "ATOMIC_POSITIONS", "NUMERICAL_DESCRIPTOR", "ABFS_ORBITAL")


def stru_sections(path) -> dict:
    """Section keyword -> token rows (the rest of the keyword's own line first)."""
    out, cur = {}, None
    for row in _rows(path):
        if row[0] in STRU_SECTIONS:
            cur = out.setdefault(row[0], [])
            if len(row) > 1:
                cur.append(row[1:])
        elif cur is not None:
            cur.append(row)
    return out


def _species(rows) -> list:
    """ATOMIC_SPECIES rows: label, mass, pseudopotential file [, type]."""
    return [(r[0], r[2]) for r in rows if len(r) >= 3]


def _positions(rows, labels):
    """ATOMIC_POSITIONS: coordinate type, then per species: label, magnetic moment, count,
    `count` coordinate rows (extra tokens are move flags)."""
    if not rows:
        raise ValueError("STRU ATOMIC_POSITIONS without a coordinate type")
    mode = rows[0][0]
    if mode not in ("Direct", "Cartesian"):
        raise NotImplementedError(f"coordinate mode {mode!r} is not provided (Direct, Cartesian)")
    it = iter(rows[1:])
    species, coords, mags = [], [], []
    try:
        for head in it:
            label = head[0]
            if label not in labels:
                raise ValueError(f"ATOMIC_POSITIONS species {label!r} is not in ATOMIC_SPECIES")
            mag = float(next(it)[0])
            count = int(float(next(it)[0]))
            for _ in range(count):
                coords.append([float(x) for x in next(it)[:3]])
                species.append(label)
                mags.append(mag)
    except StopIteration:
        raise ValueError("STRU ATOMIC_POSITIONS ends inside a species block") from None
    return mode, np.asarray(coords, dtype=np.float64).reshape(-1, 3), species, np.asarray(mags)


def read_stru(path) -> dict:
    sec = stru_sections(path)
    if "ATOMIC_POSITIONS" not in sec:
        raise ValueError("STRU without ATOMIC_POSITIONS")
    species_files = _species(sec.get("ATOMIC_SPECIES", []))
    labels = [s for s, _ in species_files]
    lat0 = float(sec["LATTICE_CONSTANT"][0][0]) if sec.get("LATTICE_CONSTANT") else 1.0
    vecs = np.asarray([[float(x) for x in r[:3]] for r in sec.get("LATTICE_VECTORS", [])[:3]], dtype=np.float64)
    if vecs.shape != (3, 3):
        raise ValueError("STRU needs three LATTICE_VECTORS rows")
    lat = vecs * lat0
    mode, c, species, mags = _positions(sec["ATOMIC_POSITIONS"], labels)
    frac = c if mode == "Direct" else (c * lat0) @ np.linalg.inv(lat)
    return dict(lattice=lat, frac=frac, species=species, magmoms=mags, labels=labels,
                pseudo_files=[f for _, f in species_files])


@dataclass
class AbacusCase:
    input: AbacusInput
    kpt: dict
    stru: dict
    psp: object

    def setup_kwargs(self) -> dict:
        from .geometry import gamma, monkhorst_pack
        args = dict(self.input.setup_args)
        if "ecut" not in args:
            raise UnmappedParameterError("INPUT has no ecutwfc")
        if self.input.tasks.get("smearing") == "fixed":
            args["sigma"] = 0.0
        args.setdefault("sigma", 0.05)
        args.setdefault("nband", 6)
        km = gamma() if self.kpt["mode"] == "gamma" else monkhorst_pack(self.kpt["mesh"], self.kpt["shift"])
        return dict(lattice=self.stru["lattice"], frac=self.stru["frac"], psp=self.psp, kmesh=km, **args)

    def system(self):
        from .api import setup
        return setup(**self.setup_kwargs())

    @property
    def scf_args(self) -> dict:
        return dict(self.input.scf_args)


def read_case(case_dir) -> AbacusCase:
    """INPUT, KPT (or kpoint_file), STRU (or stru_file) and the UPF file STRU names for the
    case's single species, under pseudo_dir."""
    from .psp import from_upf
    case = Path(case_dir)
    inp = read_input(case / "INPUT")
    kpt = read_kpt(case / inp.files.get("kpoint_file", "KPT"))
    stru = read_stru(case / inp.files.get("stru_file", "STRU"))
    if len(set(stru["species"])) != 1:
        raise NotImplementedError("one species per case (multi-species cells are rejected)")
    pfile = stru["pseudo_files"][stru["labels"].index(stru["species"][0])]
    return AbacusCase(input=inp, kpt=kpt, stru=stru, psp=from_upf(case / inp.files.get("pseudo_dir", ".") / pfile))


def setup_from_case(case_dir):
    """System of an ABACUS case directory (the reference's api.setup_from_case)."""
    return read_case(case_dir).system()
