"""UPF v1 / v2 pseudopotential reader (src/addft/geometry/upf.py:1-101).

Returns the file's arrays unconverted (Ry units for the local potential and
D; the one Ry -> Ha conversion happens in ``psp.from_upf``).  An even radial
mesh drops its last point, as ABACUS does (upf.py:44-45).
"""

from __future__ import annotations

import re
from pathlib import Path
from xml.etree import ElementTree as ET

import numpy as np

_NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[EeDd][-+]?\d+)?")


def _floats(text) -> np.ndarray:
    if text is None:
        return np.zeros(0)
    return np.asarray([float(x.replace("D", "E").replace("d", "e")) for x in _NUM.findall(text)], dtype=float)


def _block(text: str, tag: str):
    m = re.search(rf"<{tag}>(.*?)</{tag}>", text, flags=re.S)
    return m.group(1) if m else None


def _odd(n: int) -> int:
    return n - (1 if n % 2 == 0 else 0)


def _read_v2(root) -> dict:
    h = root.find("PP_HEADER")
    mesh = _odd(int(root.find("PP_MESH/PP_R").attrib["size"]))
    r = _floats(root.find("PP_MESH/PP_R").text)[:mesh]
    rab = _floats(root.find("PP_MESH/PP_RAB").text)[:mesh]
    vloc = _floats(root.find("PP_LOCAL").text)[:mesh]
    nbeta = int(h.attrib["number_of_proj"])
    lll, betar = [], []
    for ib in range(1, nbeta + 1):
        el = root.find(f"PP_NONLOCAL/PP_BETA.{ib}")
        lll.append(int(el.attrib["angular_momentum"]))
        betar.append(_floats(el.text)[:mesh])
    dij = _floats(root.find("PP_NONLOCAL/PP_DIJ").text)[:nbeta * nbeta].reshape(nbeta, nbeta)
    nlcc = h.attrib.get("core_correction", "F").strip().upper() in ("T", "TRUE", "1", ".TRUE.")
    el = root.find("PP_NLCC")
    rho_atc = _floats(el.text)[:mesh] if (nlcc and el is not None) else np.zeros(mesh)
    return dict(zval=float(h.attrib["z_valence"]), mesh=mesh, r=r, rab=rab, vloc_at=vloc, nbeta=nbeta,
                lll=np.asarray(lll, dtype=int), betar=np.asarray(betar).reshape(nbeta, mesh), dion=dij,
                nlcc=nlcc, rho_atc=rho_atc)


def _read_v1(text: str) -> dict:
    header = _block(text, "PP_HEADER")
    if header is None:
        raise ValueError("UPF v1 file without PP_HEADER")
    zval = float(re.search(r"([-\d.EeDd+]+)\s+Z valence", header).group(1).replace("D", "E"))
    mesh = _odd(int(re.search(r"(\d+)\s+Number of points in mesh", header).group(1)))
    nbeta = int(re.search(r"(\d+)\s+(\d+)\s+Number of Wavefunctions, Number of Projectors", header).group(2))
    r = _floats(_block(text, "PP_R"))[:mesh]
    rab = _floats(_block(text, "PP_RAB"))[:mesh]
    vloc = _floats(_block(text, "PP_LOCAL"))[:mesh]
    lll, betar = [], []
    for blk in re.findall(r"<PP_BETA>(.*?)</PP_BETA>", text, flags=re.S):
        v = _floats(blk)
        kb = int(v[2])
        lll.append(int(v[1]))
        b = v[3:3 + min(kb, mesh)]
        betar.append(np.pad(b, (0, mesh - len(b))))
    dv = _floats(_block(text, "PP_DIJ"))
    d = np.zeros((nbeta, nbeta))
    for k in range(int(dv[0])):
        i, j, val = int(dv[1 + 3 * k]), int(dv[2 + 3 * k]), dv[3 + 3 * k]
        d[i - 1, j - 1] = d[j - 1, i - 1] = val
    nl = _block(text, "PP_NLCC")
    return dict(zval=zval, mesh=mesh, r=r, rab=rab, vloc_at=vloc, nbeta=nbeta, lll=np.asarray(lll, dtype=int),
                betar=np.asarray(betar).reshape(nbeta, mesh), dion=d, nlcc=nl is not None,
                rho_atc=_floats(nl)[:mesh] if nl is not None else np.zeros(mesh))


def read_upf(path) -> dict:
    text = Path(path).read_text(encoding="utf-8", errors="ignore")
    if "<UPF" in text:
        return _read_v2(ET.fromstring(text))
    return _read_v1(text)
