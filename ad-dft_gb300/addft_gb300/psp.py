"""Pseudopotential description (src/addft/geometry/psp.py:19-188).

Two kinds, as the reference's ``Pseudo``:
  kind 0, synthetic(): beta_i(q) = w_i q^l_i exp(-(q b_i)^2/2) with l <= 2,
          v~_loc(q) = -amp exp(-(q sigma)^2/2), diagonal D;
  kind 1, from_upf(): radial functions from a UPF file,
          beta_i(q) = 4 pi int beta_i(r) r j_l(q r) r' dx (Simpson, psp.py:130-138),
          v~_loc(q) = 4 pi [int (r v + Z erf r) sin(q r)/q - Z exp(-q^2/4)/q^2]
          with the q = 0 value 4 pi int r (r v + Z) (psp.py:102-119).
For kind 1 the GPU kernels read the radial functions from a table on a
uniform q grid (values and exact q-derivatives, cubic Hermite in between),
built here once per pseudopotential.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

import ctypes as C
from math import erf as _erf_scalar

from . import _lib


def _erf(x):
    return np.vectorize(_erf_scalar)(x)


def _sph_j(l: int, x: np.ndarray):
    """j_l(x) and j_l'(x) for l <= 2 (psp.py:72-83), Taylor series below x = 0.1 (j_2)
    or 1e-3 (j_0, j_1); j_l' = j_(l-1) - (l+1) j_l / x."""
    small = np.abs(x) < (0.1 if l == 2 else 1e-3)
    xs = np.where(small, 1.0, x)
    s, c = np.sin(xs), np.cos(xs)
    j0 = s / xs
    if l == 0:
        j = np.where(small, 1.0 - x * x / 6.0, j0)
        dj = np.where(small, -x / 3.0 + x ** 3 / 30.0, (xs * c - s) / xs ** 2)
        return j, dj
    j1 = s / xs ** 2 - c / xs
    if l == 1:
        j = np.where(small, x / 3.0 - x ** 3 / 30.0, j1)
        dj = np.where(small, 1.0 / 3.0 - x * x / 10.0, j0 - 2.0 * j1 / xs)
        return j, dj
    if l != 2:
        raise NotImplementedError("spherical Bessel functions for l <= 2")
    j2 = (3.0 / xs ** 3 - 1.0 / xs) * s - 3.0 * c / xs ** 2
    x2 = x * x
    j = np.where(small, x2 * (1 / 15.0 - x2 * (1 / 210.0 - x2 * (1 / 7560.0 - x2 * (1 / 498960.0 - x2 / 51891840.0)))),
                 j2)
    dj = np.where(small, x * (2 / 15.0 - x2 * (4 / 210.0 - x2 * (6 / 7560.0 - x2 * (8 / 498960.0 - 10 * x2 / 51891840.0)))),
                  j1 - 3.0 * j2 / xs)
    return j, dj


@dataclass(frozen=True)
class Pseudo:
    zval: float = 2.0
    vloc_amp: float = 4.0
    vloc_sigma: float = 0.8
    proj_w: tuple = (1.0, 0.6)
    proj_b: tuple = (0.9, 1.4)
    proj_l: tuple = (0, 1)
    dion: np.ndarray = field(default_factory=lambda: np.diag([-2.0, -0.7]))
    kind: int = 0          # 0 = synthetic, 1 = UPF
    nlcc: bool = False
    r: np.ndarray = None        # kind 1: radial mesh (Bohr)
    rab: np.ndarray = None      # kind 1: dr/dx
    vloc_at: np.ndarray = None  # kind 1: v_loc(r), Ry (as in the file)
    betar: np.ndarray = None    # kind 1: (nrad, mesh) r beta(r)
    _cache: dict = field(default_factory=dict, compare=False, repr=False)

    @property
    def nspec(self) -> int:
        return 1

    @property
    def nrad(self) -> int:
        return len(self.proj_l)

    @property
    def lmax(self) -> int:
        return max(self.proj_l) if self.proj_l else 0

    @property
    def nh(self) -> int:
        return sum(2 * int(l) + 1 for l in self.proj_l)

    def lm_table(self):
        """[(radial index, l, m)] in the reference order (psp.py:57-63)."""
        return [(ib, int(l), m) for ib, l in enumerate(self.proj_l) for m in range(2 * int(l) + 1)]

    def c_struct(self) -> _lib.Psp:
        if self.nrad > 4 or any(l > 2 for l in self.proj_l):
            raise NotImplementedError("projectors with l > 2 or more than 4 radial channels")
        s = _lib.Psp()
        s.nrad = self.nrad
        s.kind = int(self.kind)
        if self.kind == 0:
            for i, (l, w, b) in enumerate(zip(self.proj_l, self.proj_w, self.proj_b)):
                s.l[i], s.w[i], s.b[i] = int(l), float(w), float(b)
            s.vloc_amp = float(self.vloc_amp)
            s.vloc_sigma = float(self.vloc_sigma)
            return s
        for i, l in enumerate(self.proj_l):
            s.l[i] = int(l)
        tab, dq, g0 = self.device_table()
        s.nq, s.dq, s.tab = int(tab.shape[-1]), float(dq), C.c_void_p(tab.data_ptr())
        s.vloc_g0 = float(g0)
        s.zval = float(self.zval)
        return s

    # -- UPF radial functions ------------------------------------------------
    QMAX, DQ = 60.0, 0.005

    def _simpson(self):
        n = self.r.shape[0]
        w = np.ones(n)
        w[1:n - 1:2] = 4.0
        w[2:n - 1:2] = 2.0
        return w / 3.0 * self.rab

    def radial(self, q):
        """(beta (nrad, nq), d beta/dq, vs (nq,), d vs/dq) at q > 0: the projectors and
        the smooth part of v~_loc, exact quadratures on the file's mesh."""
        q = np.atleast_1d(np.asarray(q, dtype=np.float64))
        r, w = self.r, self._simpson()
        x = q[:, None] * r[None, :]
        beta = np.zeros((self.nrad, q.size))
        dbeta = np.zeros_like(beta)
        for ib, l in enumerate(self.proj_l):
            f = w * self.betar[ib] * r
            jl, djl = _sph_j(int(l), x)
            beta[ib] = 4.0 * np.pi * (jl @ f)
            dbeta[ib] = 4.0 * np.pi * ((djl * r[None, :]) @ f)
        F = r * (0.5 * self.vloc_at) + self.zval * _erf(r)            # Ry -> Ha
        sn, cs = np.sin(x), np.cos(x)
        I1 = sn @ (w * F)
        I2 = cs @ (w * F * r)
        qs = np.where(q > 0, q, 1.0)
        vs = np.where(q > 0, 4.0 * np.pi * I1 / qs, np.nan)
        dvs = np.where(q > 0, 4.0 * np.pi * (I2 / qs - I1 / qs ** 2), np.nan)
        return beta, dbeta, vs, dvs

    def vloc_g0(self) -> float:
        """v~_loc(0) = 4 pi int r (r v + Z) (psp.py:117)."""
        return float(4.0 * np.pi * np.sum(self._simpson() * self.r * (self.r * 0.5 * self.vloc_at + self.zval)))

    def host_table(self):
        """(table (nrad + 1, 2, nq) f64, dq): beta_i and the smooth v~_loc with q-derivatives."""
        key = ("host", self.QMAX, self.DQ)
        if key not in self._cache:
            nq = int(np.ceil(self.QMAX / self.DQ)) + 2
            q = np.arange(nq) * self.DQ
            tab = np.zeros((self.nrad + 1, 2, nq))
            for c0 in range(1, nq, 512):
                sl = slice(c0, min(nq, c0 + 512))
                b, db, vs, dvs = self.radial(q[sl])
                tab[:self.nrad, 0, sl], tab[:self.nrad, 1, sl] = b, db
                tab[self.nrad, 0, sl], tab[self.nrad, 1, sl] = vs, dvs
            # q = 0: j_l series for the projectors; the smooth local part's limit 4 pi int r F, slope 0
            b0, db0, _, _ = self.radial(np.array([0.0]))
            tab[:self.nrad, 0, 0], tab[:self.nrad, 1, 0] = b0[:, 0], db0[:, 0]
            w = self._simpson()
            F = self.r * (0.5 * self.vloc_at) + self.zval * _erf(self.r)
            tab[self.nrad, 0, 0], tab[self.nrad, 1, 0] = 4.0 * np.pi * float(np.sum(w * F * self.r)), 0.0
            self._cache[key] = (tab, self.DQ)
        return self._cache[key]

    def device_table(self):
        key = ("device", self.QMAX, self.DQ)
        if key not in self._cache:
            import torch
            tab, dq = self.host_table()
            self._cache[key] = (torch.as_tensor(tab, device="cuda").contiguous(), dq, self.vloc_g0())
        return self._cache[key]


def synthetic(zval=(2.0,), vloc_amp=4.0, vloc_sigma=0.8, proj_w=(1.0, 0.6), proj_b=(0.9, 1.4),
              dion_diag=(-2.0, -0.7)) -> Pseudo:
    """Analytic KB pseudopotential with l = 0, 1 projectors and diagonal D (psp.py:141-164)."""
    z = zval[0] if isinstance(zval, (tuple, list)) else zval
    if isinstance(zval, (tuple, list)) and len(zval) != 1:
        raise NotImplementedError("multiple species are rejected (system.py:53-54)")
    nproj = len(proj_w)
    return Pseudo(zval=float(z), vloc_amp=float(vloc_amp), vloc_sigma=float(vloc_sigma),
                  proj_w=tuple(float(x) for x in proj_w), proj_b=tuple(float(x) for x in proj_b),
                  proj_l=tuple(range(nproj)), dion=np.diag(np.asarray(dion_diag, dtype=np.float64)))


def dion_full(psp: Pseudo, natom: int) -> np.ndarray:
    """Block-diagonal (nat*nh)^2 D with layout (i,p,j,q) (nonlocal_op.py:25-42)."""
    nh = psp.nh
    lm = psp.lm_table()
    d = np.zeros((natom, nh, natom, nh))
    for i in range(natom):
        for p, (ib, l, m) in enumerate(lm):
            for q, (jb, l2, m2) in enumerate(lm):
                if l == l2 and m == m2:
                    d[i, p, i, q] = psp.dion[ib, jb]
    return d.reshape(natom * nh, natom * nh)


def from_upf(path) -> Pseudo:
    """Pseudo (kind 1) from a UPF v1/v2 file; D converted Ry -> Ha (psp.py:167-188).
    NLCC files are rejected as in the reference."""
    from .upf import read_upf
    raw = read_upf(path)
    if raw["nlcc"]:
        raise NotImplementedError("NLCC pseudopotentials are rejected (psp.py:169-172)")
    lll = tuple(int(x) for x in raw["lll"])
    return Pseudo(zval=float(raw["zval"]), vloc_amp=0.0, vloc_sigma=1.0, proj_w=(0.0,) * len(lll),
                  proj_b=(1.0,) * len(lll), proj_l=lll, dion=np.asarray(raw["dion"], dtype=np.float64) / 2.0,
                  kind=1, nlcc=False, r=np.asarray(raw["r"]), rab=np.asarray(raw["rab"]),
                  vloc_at=np.asarray(raw["vloc_at"]), betar=np.asarray(raw["betar"]))
