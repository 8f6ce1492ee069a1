"""Pseudopotential description (src/addft/geometry/psp.py:19-164).

Only the analytic synthetic KB form is on the GPU path: beta_i(q) =
w_i q^l_i exp(-(q b_i)^2/2) with l <= 1, v~_loc(q) = -amp exp(-(q sigma)^2/2),
diagonal D.  The UPF reader of the reference is not part of this build.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib


@dataclass(frozen=True)
class Pseudo:
    zval: float = 2.0
    vloc_amp: float = 4.0
    vloc_sigma: float = 0.8
    proj_w: tuple = (1.0, 0.6)
    proj_b: tuple = (0.9, 1.4)
    proj_l: tuple = (0, 1)
    dion: np.ndarray = field(default_factory=lambda: np.diag([-2.0, -0.7]))
    kind: int = 0          # 0 = synthetic (the only kind this build supports)
    nlcc: bool = False

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
        if self.kind != 0:
            raise NotImplementedError("only the synthetic pseudopotential is supported on the GPU path")
        if self.nrad > 4 or any(l > 1 for l in self.proj_l):
            raise NotImplementedError("projectors with l > 1 or more than 4 radial channels")
        s = _lib.Psp()
        s.nrad = self.nrad
        for i, (l, w, b) in enumerate(zip(self.proj_l, self.proj_w, self.proj_b)):
            s.l[i], s.w[i], s.b[i] = int(l), float(w), float(b)
        s.vloc_amp = float(self.vloc_amp)
        s.vloc_sigma = float(self.vloc_sigma)
        return s


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
