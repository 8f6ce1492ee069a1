"""Reader of norm-conserving pseudopotential files in the Unified Pseudopotential
Format, versions 1 (tagged text) and 2 (XML).

The file is first cut into sections (``<NAME attrs> body </NAME>``, in document
order, nested sections included) by one scanner that serves both versions.  A
per-version layout then says where each field of ``UpfData`` lives:

  field      version 2 (XML)                          version 1 (tagged text)
  zval       PP_HEADER attribute z_valence            PP_HEADER line 5 ("Z valence")
  nlcc       PP_HEADER attribute core_correction      PP_HEADER line 3 ("Nonlinear Core Correction")
  nbeta      PP_HEADER attribute number_of_proj       PP_HEADER line 10, second integer
  mesh       PP_R attribute size (else header)        PP_HEADER line 9 ("Number of points in mesh")
  r, rab     PP_MESH/PP_R, PP_MESH/PP_RAB             PP_R, PP_RAB
  vloc_at    PP_LOCAL                                 PP_LOCAL
  beta_i     PP_BETA.i, l = attribute                 i-th PP_BETA: line 1 "i l", line 2 points,
             angular_momentum                         then the values (zero beyond)
  dion       PP_DIJ, nbeta x nbeta row-major          PP_DIJ: line 1 count, then "i j D_ij"
  rho_atc    PP_NLCC                                  PP_NLCC

(v1 header lines counted from 0.)  Values are returned as stored (Ry for v_loc and D); ``psp.from_upf`` converts.
A radial mesh with an even number of points loses its last point, the
convention of the reference's reader (geometry/upf.py:44-45, after ABACUS),
which keeps Simpson's rule on an odd number of points.
"""

from __future__ import annotations

import re
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_SECTION = re.compile(r"<(/?)([A-Za-z_][\w.]*)([^>]*?)(/?)>")
_ATTR = re.compile(r'([\w.]+)\s*=\s*"([^"]*)"')
_TRUE = {"t", "true", ".true.", "1", "y", "yes"}


@dataclass
class Section:
    name: str
    attrs: dict
    body: str


@dataclass
class UpfData:
    zval: float
    mesh: int
    r: np.ndarray
    rab: np.ndarray
    vloc_at: np.ndarray
    nbeta: int
    lll: np.ndarray
    betar: np.ndarray
    dion: np.ndarray
    nlcc: bool
    rho_atc: np.ndarray

    def __getitem__(self, key):
        return getattr(self, key)


def scan_sections(text: str) -> list:
    """Every tagged section of the file in document order, with its attributes and the
    raw text between its opening and closing tags ('' for self-closing tags)."""
    out, stack = [], []
    for m in _SECTION.finditer(text):
        closing, name, attrs, selfclose = m.group(1), m.group(2), m.group(3), m.group(4)
        if closing:
            for depth in range(len(stack) - 1, -1, -1):
                if stack[depth][0] == name:
                    _, a, start, slot = stack[depth]
                    out[slot] = Section(name, a, text[start:m.start()])
                    del stack[depth:]
                    break
            continue
        a = dict(_ATTR.findall(attrs))
        out.append(Section(name, a, ""))
        if not selfclose:
            stack.append((name, a, m.end(), len(out) - 1))
    return out


def numbers(text: str) -> np.ndarray:
    """All numbers of a text block; Fortran exponents (1.0D-3) accepted."""
    toks = text.replace("D", "E").replace("d", "e").split()
    vals = []
    for t in toks:
        try:
            vals.append(float(t))
        except ValueError:
            pass
    return np.asarray(vals, dtype=np.float64)


def _lines(text: str) -> list:
    return [ln for ln in text.strip().splitlines() if ln.strip()]


def _odd_mesh(n: int) -> int:
    return n if n % 2 else n - 1


def _first(sections, name):
    for s in sections:
        if s.name == name:
            return s
    return None


def _flag(word: str) -> bool:
    return word.strip().lower() in _TRUE


# ---------------------------------------------------------------------------
# version 2: metadata in attributes, arrays in element bodies
# ---------------------------------------------------------------------------
def _fields_v2(sec) -> dict:
    head = _first(sec, "PP_HEADER")
    if head is None:
        raise ValueError("UPF v2 file without PP_HEADER")
    h = head.attrs
    rsec = _first(sec, "PP_R")
    size = int(rsec.attrs.get("size", h.get("mesh_size", 0))) or numbers(rsec.body).size
    mesh = _odd_mesh(size)
    nbeta = int(h.get("number_of_proj", 0))
    betas = {}
    for s in sec:
        if s.name.startswith("PP_BETA."):
            betas[int(s.name.split(".")[1])] = s
    beta_rows, ls = [], []
    for i in range(1, nbeta + 1):
        s = betas[i]
        ls.append(int(s.attrs["angular_momentum"]))
        beta_rows.append(numbers(s.body)[:mesh])
    dij = numbers(_first(sec, "PP_DIJ").body) if nbeta else np.zeros(0)
    nlcc = _flag(h.get("core_correction", "F"))
    core = _first(sec, "PP_NLCC")
    return dict(zval=float(h["z_valence"]), mesh=mesh, nbeta=nbeta,
                r=numbers(rsec.body)[:mesh], rab=numbers(_first(sec, "PP_RAB").body)[:mesh],
                vloc_at=numbers(_first(sec, "PP_LOCAL").body)[:mesh], lll=ls, betar=beta_rows,
                dion=dij[:nbeta * nbeta].reshape(nbeta, nbeta), nlcc=nlcc,
                rho_atc=numbers(core.body)[:mesh] if (nlcc and core is not None) else np.zeros(mesh))


# ---------------------------------------------------------------------------
# version 1: a fixed-order text header, arrays in tagged blocks
# ---------------------------------------------------------------------------
# PP_HEADER lines in the order the v1 layout fixes them (value first, then a comment)
_V1_HEADER = {"nlcc": 3, "zval": 5, "mesh": 9, "counts": 10}


def _fields_v1(sec) -> dict:
    head = _first(sec, "PP_HEADER")
    if head is None:
        raise ValueError("UPF v1 file without PP_HEADER")
    lines = _lines(head.body)
    word = lambda key, k=0: lines[_V1_HEADER[key]].split()[k]  # noqa: E731
    mesh = _odd_mesh(int(word("mesh")))
    nbeta = int(word("counts", 1))
    beta_rows, ls = [], []
    for s in (s for s in sec if s.name == "PP_BETA"):
        body = _lines(s.body)
        ls.append(int(body[0].split()[1]))
        npts = int(body[1].split()[0])
        vals = numbers("\n".join(body[2:]))[:min(npts, mesh)]
        row = np.zeros(mesh)
        row[:vals.size] = vals
        beta_rows.append(row)
    dion = np.zeros((nbeta, nbeta))
    dsec = _first(sec, "PP_DIJ")
    if dsec is not None:
        body = _lines(dsec.body)
        for ln in body[1:1 + int(body[0].split()[0])]:
            i, j, val = ln.split()[:3]
            i, j = int(i) - 1, int(j) - 1
            dion[i, j] = dion[j, i] = float(val.replace("D", "E").replace("d", "e"))
    core = _first(sec, "PP_NLCC")
    return dict(zval=float(word("zval").replace("D", "E")), mesh=mesh, nbeta=nbeta,
                r=numbers(_first(sec, "PP_R").body)[:mesh], rab=numbers(_first(sec, "PP_RAB").body)[:mesh],
                vloc_at=numbers(_first(sec, "PP_LOCAL").body)[:mesh], lll=ls, betar=beta_rows, dion=dion,
                nlcc=_flag(word("nlcc")) or core is not None,
                rho_atc=numbers(core.body)[:mesh] if core is not None else np.zeros(mesh))


_LAYOUTS = {1: _fields_v1, 2: _fields_v2}


def upf_version(sections) -> int:
    top = _first(sections, "UPF")
    return 2 if top is not None else 1


def read_upf(path) -> UpfData:
    """UpfData of a UPF v1 or v2 file (values as stored: Ry, Bohr)."""
    text = Path(path).read_text(encoding="utf-8", errors="ignore")
    sec = scan_sections(text)
    f = _LAYOUTS[upf_version(sec)](sec)
    nb, mesh = f["nbeta"], f["mesh"]
    return UpfData(zval=f["zval"], mesh=mesh, r=f["r"], rab=f["rab"], vloc_at=f["vloc_at"], nbeta=nb,
                   lll=np.asarray(f["lll"], dtype=int), betar=np.asarray(f["betar"], dtype=np.float64).reshape(nb, mesh),
                   dion=np.asarray(f["dion"], dtype=np.float64), nlcc=bool(f["nlcc"]),
                   rho_atc=np.asarray(f["rho_atc"], dtype=np.float64))
