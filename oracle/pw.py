"""Oracle (test infrastructure only): plain NumPy FP64 restatement of the
ad-dft plane-wave path.

THIS MODULE IS THE CHECKER, NOT THE PRODUCT.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The GPU product (``addft_gb300``) never
imports anything under ``oracle/``.

Every function restates the reference algorithm of the file:line it cites
(paths relative to the ad-dft project root).  Conventions kept bit-for-bit
where they decide results:

* Miller ordering by |G|^2 then (m1, m2, m3) lexicographic
  (``src/addft/geometry/basis.py:118-120``);
* FFT box rule odd -> 2,3,5-smooth (``basis.py:124-132``);
* psi(r) = ifftn * N/sqrt(Omega), c_G = fftn * sqrt(Omega)/N
  (``basis.py:237-254``), n(G) = fftn/N on the *wavefunction* shell
  (``basis.py:257-262``), v(r) = N*ifftn (``basis.py:265-277``);
* structure factor e^{-iG.R}, beta carries 1/sqrt(Omega), real Ylm order
  m = 0, +1, -1 (``nonlocal_op.py:45-64``, ``ylm.py:8-26``);
* PZ81 with rho clamped at 1e-14 (``xc.py:139-161``).

Parity of this oracle with the reference JAX FP64 path is pinned by the
reference's own recorded numbers (fixture energy -2.57875 Ha,
``docs/ARCHITECTURE.md:295``) and by its known-answer tests (Hartree
plane-wave exactness, UEG, two energy forms, force vs central FD), which
``tests/test_oracle_*.py`` re-run against this module.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass, field, replace
from math import erfc as _erfc_scalar

import numpy as np

FOUR_PI = 4.0 * np.pi
HA_TO_KBAR = 2.942105e5  # src/addft/runtime/units.py:16


# ----------------------------------------------------------------------------
# Cell / k-mesh   (src/addft/geometry/cell.py:17-59, kmesh.py:19-59)
# ----------------------------------------------------------------------------

def reciprocal(lattice):
    """B = 2 pi inv(L)^T, rows b1,b2,b3 (cell.py:28-30)."""
    return 2.0 * np.pi * np.linalg.inv(np.asarray(lattice, dtype=float)).T


def volume(lattice):
    return abs(float(np.linalg.det(np.asarray(lattice, dtype=float))))


def positions(lattice, frac):
    return np.asarray(frac, dtype=float) @ np.asarray(lattice, dtype=float)


def strained(lattice, eps):
    """L' = L (I + eps), fractional coordinates fixed (cell.py:46-53)."""
    return np.asarray(lattice, dtype=float) @ (np.eye(3) + np.asarray(eps, dtype=float))


@dataclass
class KMesh:
    kfrac: np.ndarray
    weights: np.ndarray

    def cartesian(self, lattice):
        return self.kfrac @ reciprocal(lattice)


def gamma():
    return KMesh(np.zeros((1, 3)), np.ones(1))


def monkhorst_pack(n, shift=None):
    """MP grid folded into [-0.5, 0.5) with equal weights (kmesh.py:33-55)."""
    n = tuple(int(x) for x in n)
    shift = (0.0, 0.0, 0.0) if shift is None else tuple(float(x) for x in shift)
    pts = [((i + shift[0]) / n[0], (j + shift[1]) / n[1], (k + shift[2]) / n[2])
           for i in range(n[0]) for j in range(n[1]) for k in range(n[2])]
    frac = np.asarray(pts, dtype=float)
    frac = np.where(frac >= 0.5, frac - 1.0, frac)
    return KMesh(frac, np.full(frac.shape[0], 1.0 / frac.shape[0]))


# ----------------------------------------------------------------------------
# Basis / FFT box   (src/addft/geometry/basis.py:59-144)
# ----------------------------------------------------------------------------

def is_smooth235(n):
    if n < 1:
        return False
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


def smooth_up(n):
    while not is_smooth235(n):
        n += 1
    return n


def _nmax_on_axis(lattice, gcut2, kmax=0.0):
    lat = np.asarray(lattice, dtype=float)
    a_len = np.linalg.norm(lat, axis=1)
    m = np.ceil((np.sqrt(gcut2) + kmax) * a_len / (2.0 * np.pi)).astype(int)
    return int(m[0]), int(m[1]), int(m[2])


def build_miller(lattice, ecut, kpts=None):
    """Frozen union shell |k+G|^2 <= 2 ecut, sorted by |G|^2 then m (basis.py:89-121)."""
    gcut2 = 2.0 * float(ecut)
    lat = np.asarray(lattice, dtype=float)
    bmat = 2.0 * np.pi * np.linalg.inv(lat).T
    ks = np.zeros((1, 3)) if kpts is None else np.asarray(kpts, dtype=float)
    kmax = float(np.max(np.linalg.norm(ks, axis=1)))
    m1, m2, m3 = _nmax_on_axis(lattice, gcut2, kmax)
    rng = np.stack(np.meshgrid(np.arange(-m1, m1 + 1), np.arange(-m2, m2 + 1),
                               np.arange(-m3, m3 + 1), indexing="ij"), axis=-1).reshape(-1, 3)
    bmat_inv = np.linalg.inv(bmat)
    keep = np.zeros(len(rng), dtype=bool)
    for k in ks:
        kfrac = k @ bmat_inv
        cart = (rng + kfrac) @ bmat
        keep |= np.sum(cart ** 2, axis=1) <= gcut2 * (1.0 + 1e-12)
    miller = rng[keep]
    g2 = np.sum((miller @ bmat) ** 2, axis=1)
    order = np.lexsort((miller[:, 2], miller[:, 1], miller[:, 0], g2))
    return miller[order].astype(np.int32)


def fft_shape(lattice, ecut, density_factor=4.0):
    """Odd box 2m+1 rounded up to 2,3,5-smooth (basis.py:124-132)."""
    gcut2 = 2.0 * float(ecut) * float(density_factor)
    return tuple(smooth_up(2 * m + 1) for m in _nmax_on_axis(lattice, gcut2))


@dataclass
class Basis:
    miller: np.ndarray
    ecut: float
    fft_shape: tuple
    miller_rho: np.ndarray

    @property
    def nG(self):
        return int(self.miller.shape[0])

    @property
    def nfft(self):
        return int(np.prod(self.fft_shape))


def make_basis(lattice, ecut, density_factor=4.0, kpts=None):
    """basis.py:135-144."""
    return Basis(miller=build_miller(lattice, ecut, kpts=kpts), ecut=float(ecut),
                 fft_shape=fft_shape(lattice, ecut, density_factor),
                 miller_rho=build_miller(lattice, float(ecut) * float(density_factor)))


def gvectors(miller, lattice, kpoint=None):
    g = miller.astype(float) @ reciprocal(lattice)
    if kpoint is not None:
        g = g + np.asarray(kpoint, dtype=float)[None, :]
    return g


def safe_norm(v, eps=1e-30):
    r2 = np.sum(v * v, axis=-1)
    return np.where(r2 > eps, np.sqrt(np.where(r2 > eps, r2, 1.0)), 0.0)


def flat_index(shape, miller):
    """((m1 mod n1) n2 + m2 mod n2) n3 + m3 mod n3 (basis.py:196-202)."""
    n1, n2, n3 = shape
    m = np.asarray(miller)
    return ((np.mod(m[:, 0], n1) * n2 + np.mod(m[:, 1], n2)) * n3
            + np.mod(m[:, 2], n3)).astype(np.int64)


def coeffs_to_grid(shape, c, miller):
    lead = c.shape[:-1]
    flat = np.zeros(lead + (int(np.prod(shape)),), dtype=c.dtype)
    flat[..., flat_index(shape, miller)] = c
    return flat.reshape(lead + tuple(shape))


def grid_to_coeffs(shape, arr, miller):
    lead = arr.shape[:-3]
    return arr.reshape(lead + (-1,))[..., flat_index(shape, miller)]


def psi_to_real(basis, lattice, c):
    """psi(r) = ifftn(scatter c) * N/sqrt(Omega), flattened (basis.py:237-244)."""
    n = basis.nfft
    grid = coeffs_to_grid(basis.fft_shape, np.asarray(c), basis.miller)
    out = np.fft.ifftn(grid, axes=(-3, -2, -1)) * (n / np.sqrt(volume(lattice)))
    return out.reshape(np.asarray(c).shape[:-1] + (n,))


def real_to_psi(basis, lattice, psi_r):
    """c_G = gather(fftn(psi_r)) * sqrt(Omega)/N (basis.py:247-254)."""
    n = basis.nfft
    grid = np.asarray(psi_r).reshape(np.asarray(psi_r).shape[:-1] + tuple(basis.fft_shape))
    spec = np.fft.fftn(grid, axes=(-3, -2, -1)) * (np.sqrt(volume(lattice)) / n)
    return grid_to_coeffs(basis.fft_shape, spec, basis.miller)


def density_g(basis, rho_r):
    """n(G) = fftn(rho)/N on the wavefunction shell (basis.py:257-262)."""
    spec = np.fft.fftn(np.asarray(rho_r).reshape(basis.fft_shape)) / basis.nfft
    return grid_to_coeffs(basis.fft_shape, spec, basis.miller)


def real_from_g(basis, vg, miller=None):
    """v(r) = Re(N ifftn(scatter vg)) (basis.py:265-277)."""
    miller = basis.miller if miller is None else miller
    grid = coeffs_to_grid(basis.fft_shape, np.asarray(vg, dtype=complex), miller)
    return (basis.nfft * np.fft.ifftn(grid)).real.reshape(basis.nfft)


# ----------------------------------------------------------------------------
# Pseudopotential (synthetic KB), Ylm   (psp.py:57-164, ylm.py:8-26)
# ----------------------------------------------------------------------------

@dataclass
class Pseudo:
    """KB pseudopotential, one species: kind 0 synthetic analytic (psp.py:141-164),
    kind 1 from a UPF file (psp.py:102-138, 167-188)."""
    zval: float = 2.0
    vloc_amp: float = 4.0
    vloc_sigma: float = 0.8
    proj_w: tuple = (1.0, 0.6)
    proj_b: tuple = (0.9, 1.4)
    proj_l: tuple = (0, 1)
    dion: np.ndarray = field(default_factory=lambda: np.diag([-2.0, -0.7]))
    kind: int = 0
    r: np.ndarray = None
    rab: np.ndarray = None
    vloc_at: np.ndarray = None      # Ry, as in the file
    betar: np.ndarray = None

    @property
    def lmax(self):
        return max(self.proj_l)

    @property
    def nh(self):
        return sum(2 * l + 1 for l in self.proj_l)

    def lm_table(self):
        """[(radial index, l, m)] with m = 0..2l (psp.py:57-63)."""
        return [(ib, int(l), m) for ib, l in enumerate(self.proj_l) for m in range(2 * int(l) + 1)]


def synthetic(zval=2.0, vloc_amp=4.0, vloc_sigma=0.8, proj_w=(1.0, 0.6),
              proj_b=(0.9, 1.4), dion_diag=(-2.0, -0.7)):
    nproj = len(proj_w)
    return Pseudo(zval=float(zval), vloc_amp=float(vloc_amp), vloc_sigma=float(vloc_sigma),
                  proj_w=tuple(float(x) for x in proj_w), proj_b=tuple(float(x) for x in proj_b),
                  proj_l=tuple(range(nproj)), dion=np.diag(np.asarray(dion_diag, dtype=float)))


# -- UPF radial functions: Simpson on the file's mesh at every q (psp.py:66-138) --
def read_upf(path):
    """UPF v2 (XML) or v1 (text) arrays, unconverted; even meshes drop their last
    point (upf.py:40-95)."""
    import re
    from pathlib import Path
    from xml.etree import ElementTree as ET
    num = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[EeDd][-+]?\d+)?")

    def fl(t):
        return np.asarray([float(x.replace("D", "E")) for x in num.findall(t or "")])

    text = Path(path).read_text()
    if "<UPF" in text:
        root = ET.fromstring(text)
        h = root.find("PP_HEADER")
        mesh = int(root.find("PP_MESH/PP_R").attrib["size"])
        mesh -= 1 if mesh % 2 == 0 else 0
        nb = int(h.attrib["number_of_proj"])
        betas = [root.find(f"PP_NONLOCAL/PP_BETA.{i}") for i in range(1, nb + 1)]
        return dict(zval=float(h.attrib["z_valence"]), r=fl(root.find("PP_MESH/PP_R").text)[:mesh],
                    rab=fl(root.find("PP_MESH/PP_RAB").text)[:mesh], vloc_at=fl(root.find("PP_LOCAL").text)[:mesh],
                    lll=[int(b.attrib["angular_momentum"]) for b in betas],
                    betar=np.stack([fl(b.text)[:mesh] for b in betas]),
                    dion=fl(root.find("PP_NONLOCAL/PP_DIJ").text)[:nb * nb].reshape(nb, nb))
    blk = lambda tag: re.search(rf"<{tag}>(.*?)</{tag}>", text, flags=re.S).group(1)  # noqa: E731
    head = blk("PP_HEADER")
    mesh = int(re.search(r"(\d+)\s+Number of points in mesh", head).group(1))
    mesh -= 1 if mesh % 2 == 0 else 0
    lll, betar = [], []
    for b in re.findall(r"<PP_BETA>(.*?)</PP_BETA>", text, flags=re.S):
        v = fl(b)
        lll.append(int(v[1]))
        betar.append(np.pad(v[3:3 + min(int(v[2]), mesh)], (0, max(0, mesh - min(int(v[2]), mesh)))))
    dv = fl(blk("PP_DIJ"))
    d = np.zeros((len(lll), len(lll)))
    for k in range(int(dv[0])):
        i, j = int(dv[1 + 3 * k]) - 1, int(dv[2 + 3 * k]) - 1
        d[i, j] = d[j, i] = dv[3 + 3 * k]
    return dict(zval=float(re.search(r"([-\d.EeDd+]+)\s+Z valence", head).group(1)), r=fl(blk("PP_R"))[:mesh],
                rab=fl(blk("PP_RAB"))[:mesh], vloc_at=fl(blk("PP_LOCAL"))[:mesh], lll=lll, betar=np.stack(betar),
                dion=d)


def from_upf(path):
    """Pseudo kind 1, D in Ha (psp.py:167-188)."""
    raw = read_upf(path)
    n = len(raw["lll"])
    return Pseudo(zval=raw["zval"], vloc_amp=0.0, vloc_sigma=1.0, proj_w=(0.0,) * n, proj_b=(1.0,) * n,
                  proj_l=tuple(raw["lll"]), dion=raw["dion"] / 2.0, kind=1, r=raw["r"], rab=raw["rab"],
                  vloc_at=raw["vloc_at"], betar=raw["betar"])


def _simpson_w(psp):
    n = psp.r.shape[0]
    w = np.ones(n)
    w[1:n - 1:2] = 4.0
    w[2:n - 1:2] = 2.0
    return w / 3.0 * psp.rab


def _sph_jl(l, x):
    """j_l and j_l' for l <= 2 (psp.py:72-83; the derivative by the recurrence
    j_l' = j_(l-1) - (l+1) j_l / x; Taylor series at small x)."""
    xs = np.where(np.abs(x) > 1e-4, x, 1.0)
    if l == 0:
        j = np.where(np.abs(x) > 1e-4, np.sin(xs) / xs, 1.0 - x * x / 6.0)
        dj = np.where(np.abs(x) > 1e-4, (xs * np.cos(xs) - np.sin(xs)) / xs ** 2, -x / 3.0)
        return j, dj
    j1 = np.where(np.abs(x) > 1e-4, np.sin(xs) / xs ** 2 - np.cos(xs) / xs, x / 3.0)
    j0 = np.where(np.abs(x) > 1e-4, np.sin(xs) / xs, 1.0 - x * x / 6.0)
    if l == 1:
        dj = np.where(np.abs(x) > 1e-4, j0 - 2.0 * j1 / xs, 1.0 / 3.0 - x * x / 10.0)
        return j1, dj
    if l != 2:
        raise NotImplementedError("spherical Bessel functions for l <= 2 (psp.py:72-83)")
    # series sum_k (-x^2/2)^k x^2 / (k! 15 * 7 * 9 * ... (2k + 5)) below x = 0.1
    big = np.abs(x) > 0.1
    xb = np.where(big, x, 1.0)
    ser, dser, term = np.zeros_like(x), np.zeros_like(x), x * x / 15.0
    for k in range(6):
        ser = ser + term
        dser = dser + (2 * k + 2) * term / np.where(big, 1.0, np.where(x == 0, 1.0, x))
        term = term * (-x * x / 2.0) / ((k + 1) * (2 * k + 7))
    dser = np.where(x == 0, 0.0, dser)
    j2 = np.where(big, (3.0 / xb ** 3 - 1.0 / xb) * np.sin(xb) - 3.0 * np.cos(xb) / xb ** 2, ser)
    j1b = np.where(big, np.sin(xb) / xb ** 2 - np.cos(xb) / xb, 0.0)
    dj = np.where(big, j1b - 3.0 * j2 / xb, dser)
    return j2, dj


def _upf_local_parts(psp, q):
    from math import erf
    r, w = psp.r, _simpson_w(psp)
    F = r * (psp.vloc_at / 2.0) + psp.zval * np.array([erf(x) for x in r])
    qs = np.where(q > 1e-12, q, 1.0)
    x = qs[..., None] * r
    i1 = np.sum(w * F * np.sin(x), axis=-1)
    i2 = np.sum(w * F * r * np.cos(x), axis=-1)
    g0 = FOUR_PI * np.sum(w * r * (r * psp.vloc_at / 2.0 + psp.zval))
    return qs, i1, i2, g0


def vloc_q(psp, q):
    """v~(q): kind 0 -amp exp(-(q sigma)^2/2) (psp.py:92-95); kind 1 the UPF transform
    4 pi [int (r v + Z erf r) sin(q r)/q - Z exp(-q^2/4)/q^2], q = 0: 4 pi int r (r v + Z)
    (psp.py:102-119)."""
    if psp.kind == 0:
        return -psp.vloc_amp * np.exp(-0.5 * (q * psp.vloc_sigma) ** 2)
    q = np.asarray(q, dtype=float)
    qs, i1, _, g0 = _upf_local_parts(psp, q)
    v = FOUR_PI * (i1 / qs - psp.zval * np.exp(-qs ** 2 / 4.0) / qs ** 2)
    return np.where(q > 1e-12, v, g0)


def vloc_q_deriv(psp, q):
    if psp.kind == 0:
        return -q * psp.vloc_sigma ** 2 * vloc_q(psp, q)
    q = np.asarray(q, dtype=float)
    qs, i1, i2, _ = _upf_local_parts(psp, q)
    e = psp.zval * np.exp(-qs ** 2 / 4.0)
    d = FOUR_PI * (i2 / qs - i1 / qs ** 2 + e * (0.5 / qs + 2.0 / qs ** 3))
    return np.where(q > 1e-12, d, 0.0)


def _upf_beta(psp, q, deriv):
    r, w = psp.r, _simpson_w(psp)
    q = np.asarray(q, dtype=float)
    out = []
    for ib, l in enumerate(psp.proj_l):
        j, dj = _sph_jl(int(l), q[..., None] * r)
        f = w * psp.betar[ib] * r
        out.append(FOUR_PI * np.sum(f * (dj * r if deriv else j), axis=-1))
    return np.stack(out, axis=0)


def beta_q(psp, q):
    """beta_i(q): kind 0 w q^l exp(-(q b)^2/2) clamped at 1e-12 (psp.py:122-128); kind 1
    4 pi int beta_i(r) r j_l(q r) (psp.py:130-138)."""
    if psp.kind == 1:
        return _upf_beta(psp, q, False)
    qq = np.maximum(q, 1e-12)
    return np.stack([w * qq ** l * np.exp(-0.5 * (qq * b) ** 2)
                     for w, b, l in zip(psp.proj_w, psp.proj_b, psp.proj_l)], axis=0)


def beta_q_deriv(psp, q):
    """d beta_i / dq (kind 0: zero below the 1e-12 clamp, like the reference's AD)."""
    if psp.kind == 1:
        return _upf_beta(psp, q, True)
    qq = np.maximum(q, 1e-12)
    act = (q > 1e-12).astype(float)
    out = []
    for w, b, l in zip(psp.proj_w, psp.proj_b, psp.proj_l):
        e = np.exp(-0.5 * (qq * b) ** 2)
        d = w * e * ((l * qq ** (l - 1) if l > 0 else 0.0) - qq ** (l + 1) * b * b)
        out.append(d * act)
    return np.stack(out, axis=0)


def ylm_real(lmax, g):
    """Real Ylm, l<=2, ABACUS order m = 0,+1,-1,+2,-2 (ylm.py:8-26)."""
    g = np.asarray(g, dtype=float)
    x, y, z = g[..., 0], g[..., 1], g[..., 2]
    r2 = np.sum(g * g, axis=-1)
    rs = np.sqrt(np.where(r2 > 1e-30, r2, 1.0))
    out = [np.ones_like(rs) / np.sqrt(FOUR_PI)]
    if lmax >= 1:
        c1 = np.sqrt(3.0 / FOUR_PI) / rs
        out += [c1 * z, -c1 * x, -c1 * y]
    if lmax >= 2:
        out += [np.sqrt(5.0 / FOUR_PI) * (3.0 * z * z - r2) / (2.0 * rs * rs),
                -np.sqrt(15.0 / FOUR_PI) * x * z / (rs * rs),
                -np.sqrt(15.0 / FOUR_PI) * y * z / (rs * rs),
                np.sqrt(15.0 / (16.0 * np.pi)) * (x * x - y * y) / (rs * rs),
                np.sqrt(15.0 / FOUR_PI) * x * y / (rs * rs)]
    return np.stack(out, axis=-1)


def ylm_real_grad(lmax, g):
    """d Y_lm / d g_c, shape (..., (lmax+1)^2, 3), for l <= 2 (zero at g = 0).  The l = 2
    functions are P(g) / r^2 with P quadratic (ylm.py:18-25), so
    dY/dg_c = (dP/dg_c) / r^2 - 2 P g_c / r^4."""
    if lmax > 2:
        raise NotImplementedError("projector derivatives implemented for l <= 2")
    g = np.asarray(g, dtype=float)
    r2 = np.sum(g * g, axis=-1)
    pos = r2 > 1e-30
    rs = np.sqrt(np.where(pos, r2, 1.0))
    out = np.zeros(g.shape[:-1] + ((lmax + 1) ** 2, 3))
    if lmax >= 1:
        c1 = np.sqrt(3.0 / FOUR_PI)
        u = g / rs[..., None]
        # d(u_c)/d g_a = (delta_ca - u_c u_a)/r
        eye = np.eye(3)
        du = (eye[None, :, :] - u[..., :, None] * u[..., None, :]) / rs[..., None, None]
        du = np.where(pos[..., None, None], du, 0.0)
        out[..., 1, :] = c1 * du[..., 2, :]
        out[..., 2, :] = -c1 * du[..., 0, :]
        out[..., 3, :] = -c1 * du[..., 1, :]
    if lmax >= 2:
        x, y, z = g[..., 0], g[..., 1], g[..., 2]
        zero = np.zeros_like(x)
        c20, c2, c22 = np.sqrt(5.0 / FOUR_PI), np.sqrt(15.0 / FOUR_PI), np.sqrt(15.0 / (16.0 * np.pi))
        # Y = P / r^2 with P and its gradient (dP/dx, dP/dy, dP/dz)
        polys = [(c20 * (3.0 * z * z - r2) / 2.0, (-c20 * x, -c20 * y, 2.0 * c20 * z)),
                 (-c2 * x * z, (-c2 * z, zero, -c2 * x)),
                 (-c2 * y * z, (zero, -c2 * z, -c2 * y)),
                 (c22 * (x * x - y * y), (2.0 * c22 * x, -2.0 * c22 * y, zero)),
                 (c2 * x * y, (c2 * y, c2 * x, zero))]
        rr = rs * rs
        for j, (P, dP) in enumerate(polys):
            for c in range(3):
                v = dP[c] / rr - 2.0 * P * g[..., c] / (rr * rr)
                out[..., 4 + j, c] = np.where(pos, v, 0.0)
    return out


# ----------------------------------------------------------------------------
# Static / state   (src/addft/system.py:24-69)
# ----------------------------------------------------------------------------

@dataclass
class Static:
    basis: Basis
    kpts: np.ndarray
    kweights: np.ndarray
    psp: Pseudo
    natom: int
    nband: int
    spin_degeneracy: float
    sigma: float
    nelec: float
    eta_ewald: float


@dataclass
class SCFState:
    psi: np.ndarray
    eig: np.ndarray
    occ: np.ndarray
    mu: float
    rho_r: np.ndarray
    n_iter: int
    residual: float


@dataclass
class System:
    lattice: np.ndarray
    frac: np.ndarray
    static: Static


def setup(lattice, frac, psp=None, ecut=8.0, nband=4, kmesh=None, sigma=0.05,
          density_factor=4.0, eta_ewald=0.9):
    """api.py:35-45 + system.py:47-69 (sigma default 0.05 through setup)."""
    lattice = np.asarray(lattice, dtype=float)
    frac = np.asarray(frac, dtype=float)
    psp = synthetic() if psp is None else psp
    kmesh = kmesh or gamma()
    kpts = kmesh.cartesian(lattice)
    basis = make_basis(lattice, ecut, density_factor, kpts=kpts)
    natom = frac.shape[0]
    static = Static(basis=basis, kpts=kpts, kweights=np.asarray(kmesh.weights, dtype=float),
                    psp=psp, natom=natom, nband=int(nband), spin_degeneracy=2.0,
                    sigma=float(sigma), nelec=float(psp.zval * natom), eta_ewald=float(eta_ewald))
    return System(lattice=lattice, frac=frac, static=static)


# ----------------------------------------------------------------------------
# Physics primitives
# ----------------------------------------------------------------------------

def local_potential_g(static, lattice, frac):
    """V_loc(G) = (1/Omega) sum_I v~(|G|) e^{-iG.R_I} on miller_rho (local.py:21-33)."""
    g = gvectors(static.basis.miller_rho, lattice)
    q = safe_norm(g)
    amp = vloc_q(static.psp, q)
    r = positions(lattice, frac)
    sf = np.sum(np.exp(-1j * (g @ r.T)), axis=-1)
    return amp * sf / volume(lattice)


def local_potential_r(static, lattice, frac):
    return real_from_g(static.basis, local_potential_g(static, lattice, frac),
                       static.basis.miller_rho)


def dion_full(psp, natom):
    """Block-diagonal D, layout (i,p,j,q) (nonlocal_op.py:25-42)."""
    nh = psp.nh
    lm = psp.lm_table()
    d = np.zeros((natom, nh, natom, nh))
    for i in range(natom):
        for p, (ib, l, m) in enumerate(lm):
            for q_, (jb, l2, m2) in enumerate(lm):
                if l == l2 and m == m2:
                    d[i, p, i, q_] = psp.dion[ib, jb]
    return d.reshape(natom * nh, natom * nh)


def projectors(static, lattice, frac):
    """(nk, nat*nh, nG): beta(|k+G|) Y_lm(k+G) e^{-i(k+G).R}/sqrt(Omega) (nonlocal_op.py:45-64)."""
    psp, basis = static.psp, static.basis
    r = positions(lattice, frac)
    omega = volume(lattice)
    out = []
    for k in static.kpts:
        gk = gvectors(basis.miller, lattice, k)
        q = safe_norm(gk)
        ylm = ylm_real(psp.lmax, gk)
        phase = np.exp(-1j * (gk @ r.T))
        bet = beta_q(psp, q)
        rows = []
        for i in range(r.shape[0]):
            for ib, l, m in psp.lm_table():
                rows.append(bet[ib] * ylm[:, l * l + m] * phase[:, i])
        out.append(np.stack(rows, axis=0) / np.sqrt(omega))
    return np.stack(out, axis=0)


def becp(proj, psi):
    """<beta|psi>: (nk,P,nG),(nk,nb,nG) -> (nk,P,nb) (nonlocal_op.py:67-69)."""
    return np.einsum("kpg,kng->kpn", np.conj(proj), psi)


def vnl_apply(proj, dion, psi):
    """beta D <beta|psi> (nonlocal_op.py:72-76)."""
    b = becp(proj, psi)
    return np.einsum("kpg,kpn->kng", proj, np.einsum("pq,kqn->kpn", dion, b))


def nonlocal_energy(proj, dion, psi, occ, weights, spin_degeneracy=2.0):
    """nonlocal_op.py:79-82."""
    b = becp(proj, psi)
    e = np.einsum("kpn,pq,kqn->kn", np.conj(b), dion, b).real
    return float(np.sum(weights[:, None] * occ * e) * spin_degeneracy)


def density_from_psi(basis, lattice, psi, occ, weights, spin_degeneracy=2.0):
    """rho(r) = sum_k,b w_k f_kb g_s |psi_kb(r)|^2 (density.py:18-23)."""
    psi_r = psi_to_real(basis, lattice, psi)
    w = weights[:, None] * occ * spin_degeneracy
    return np.einsum("kb,kbi->i", w, (psi_r * np.conj(psi_r)).real)


def _vh_g(basis, lattice, rho_r):
    ng = density_g(basis, rho_r)
    q2 = np.sum(gvectors(basis.miller, lattice) ** 2, axis=-1)
    safe = np.where(q2 > 1e-14, q2, 1.0)
    vg = np.where(q2 > 1e-14, FOUR_PI * ng / safe, 0.0)
    return vg, ng, q2


def hartree_energy(basis, lattice, rho_r):
    """E_H = Omega/2 sum Re(n V*) (hartree.py:21-32)."""
    vg, ng, q2 = _vh_g(basis, lattice, rho_r)
    return float(0.5 * volume(lattice) * np.sum(np.where(q2 > 1e-14, (ng * np.conj(vg)).real, 0.0)))


def hartree_potential_r(basis, lattice, rho_r):
    """hartree.py:35-48 (V_G stays complex)."""
    vg, _, _ = _vh_g(basis, lattice, rho_r)
    return real_from_g(basis, vg)


# --- LDA PZ81 (xc.py:51-73) with analytic first/second derivatives ---------
_A, _B, _C, _D = 0.0311, -0.048, 0.0020, -0.0116
_G, _B1, _B2 = -0.1423, 1.0529, 0.3334
RHO_MIN = 1e-14


def eps_x(n):
    n = np.maximum(n, RHO_MIN)
    return -(3.0 / 4.0) * np.power(3.0 * n / np.pi, 1.0 / 3.0)


def _rs(n):
    return np.power(3.0 / (4.0 * np.pi * np.maximum(n, RHO_MIN)), 1.0 / 3.0)


def eps_c(n):
    rs = _rs(n)
    small = _A * np.log(rs) + _B + _C * rs * np.log(rs) + _D * rs
    large = _G / (1.0 + _B1 * np.sqrt(rs) + _B2 * rs)
    return np.where(rs < 1.0, small, large)


def _deps_c_drs(rs):
    small = _A / rs + _C * (np.log(rs) + 1.0) + _D
    den = 1.0 + _B1 * np.sqrt(rs) + _B2 * rs
    large = -_G * (0.5 * _B1 / np.sqrt(rs) + _B2) / den ** 2
    return np.where(rs < 1.0, small, large)


def _d2eps_c_drs2(rs):
    small = -_A / rs ** 2 + _C / rs
    den = 1.0 + _B1 * np.sqrt(rs) + _B2 * rs
    dp = 0.5 * _B1 / np.sqrt(rs) + _B2
    dpp = -0.25 * _B1 / rs ** 1.5
    large = -_G * dpp / den ** 2 + 2.0 * _G * dp ** 2 / den ** 3
    return np.where(rs < 1.0, small, large)


def lda_x_energy_density(n):
    return np.maximum(n, RHO_MIN) * eps_x(n)


def lda_c_energy_density(n):
    return np.maximum(n, RHO_MIN) * eps_c(n)


def lda_energy_density(n):
    return np.maximum(n, RHO_MIN) * (eps_x(n) + eps_c(n))


def xc_potential_point(n):
    """v = d[n eps]/dn; zero below the clamp, as jax.grad through max() gives (xc.py:152-173)."""
    n = np.asarray(n, dtype=float)
    rs = _rs(n)
    vx = (4.0 / 3.0) * eps_x(n)
    vc = eps_c(n) - (rs / 3.0) * _deps_c_drs(rs)
    return np.where(n > RHO_MIN, vx + vc, 0.0)


def xc_kernel_point(n):
    """f_xc = d^2[n eps]/dn^2 (xc.py:176-191)."""
    n = np.asarray(n, dtype=float)
    nn = np.maximum(n, RHO_MIN)
    rs = _rs(n)
    fx = (4.0 / 9.0) * eps_x(n) / nn
    fc = ((2.0 / 3.0) * _deps_c_drs(rs) - (rs / 3.0) * _d2eps_c_drs2(rs)) * (-rs / (3.0 * nn))
    return np.where(n > RHO_MIN, fx + fc, 0.0)


def native_xc_lda(rho):
    """The reference's fused native XC handler (native/xc_lda.cu:28-45): v_xc and
    sum n (eps_x + eps_c) both at the clamped density max(rho, 1e-14) -- unlike the
    analytic path, v_xc is not zeroed below the clamp."""
    n = np.maximum(np.asarray(rho, dtype=float), RHO_MIN)
    rs = _rs(n)
    vxc = (4.0 / 3.0) * eps_x(n) + eps_c(n) - (rs / 3.0) * _deps_c_drs(rs)
    return vxc, float(np.sum(n * (eps_x(n) + eps_c(n))))


def xc_energy_lda(basis, lattice, rho_r):
    return float(volume(lattice) / basis.nfft * np.sum(lda_energy_density(rho_r)))


def exchange_energy_lda(basis, lattice, rho_r):
    return float(volume(lattice) / basis.nfft * np.sum(lda_x_energy_density(rho_r)))


def correlation_energy_lda(basis, lattice, rho_r):
    return float(volume(lattice) / basis.nfft * np.sum(lda_c_energy_density(rho_r)))


# --- Ewald (ewald.py:34-77) -------------------------------------------------
_erfc = np.vectorize(_erfc_scalar)


def _ewald_parts(lattice, frac, charges, eta, nmax):
    lat = np.asarray(lattice, dtype=float)
    r = positions(lat, frac)
    trans = np.asarray(list(itertools.product(range(-nmax, nmax + 1), repeat=3)), dtype=float)
    tvec = trans @ lat
    zero = np.all(trans == 0, axis=-1)
    bmat = reciprocal(lat)
    m = np.asarray(list(itertools.product(range(-nmax - 2, nmax + 3), repeat=3)), dtype=float)
    g = m @ bmat
    g2 = np.sum(g * g, axis=-1)
    keep = g2 > 1e-12
    return r, tvec, zero, g, g2, keep


def ewald_energy(lattice, frac, charges, eta=0.9, nmax=8):
    lat = np.asarray(lattice, dtype=float)
    z = np.asarray(charges, dtype=float)
    omega = volume(lat)
    r, tvec, zero, g, g2, keep = _ewald_parts(lat, frac, z, eta, nmax)
    nat = len(z)
    e_real = 0.0
    for i in range(nat):
        for j in range(nat):
            d = r[i] - r[j] + tvec
            dist = np.sqrt(np.sum(d * d, axis=-1) + 1e-30)
            val = _erfc(eta * dist) / dist
            if i == j:
                val = np.where(zero, 0.0, val)
            e_real += 0.5 * z[i] * z[j] * np.sum(val)
    g2s = np.where(keep, g2, 1.0)
    sf = np.sum(z[None, :] * np.exp(-1j * (g @ r.T)), axis=-1)
    term = np.where(keep, np.exp(-g2s / (4.0 * eta ** 2)) / g2s * (sf * np.conj(sf)).real, 0.0)
    e_recip = 2.0 * np.pi / omega * np.sum(term)
    e_self = -(eta / np.sqrt(np.pi)) * np.sum(z * z)
    e_bg = -(np.pi / (2.0 * omega * eta ** 2)) * np.sum(z) ** 2
    return float(e_real + e_recip + e_self + e_bg)


def ewald_gradients(lattice, frac, charges, eta=0.9, nmax=8):
    """(dE/dR (nat,3), dE/deps (3,3)) of ewald_energy, analytic."""
    lat = np.asarray(lattice, dtype=float)
    z = np.asarray(charges, dtype=float)
    omega = volume(lat)
    r, tvec, zero, g, g2, keep = _ewald_parts(lat, frac, z, eta, nmax)
    nat = len(z)
    dR = np.zeros((nat, 3))
    deps = np.zeros((3, 3))
    e_real = 0.0
    for i in range(nat):
        for j in range(nat):
            d = r[i] - r[j] + tvec
            dist = np.sqrt(np.sum(d * d, axis=-1) + 1e-30)
            phi = _erfc(eta * dist) / dist
            dphi = -phi / dist - (2.0 * eta / np.sqrt(np.pi)) * np.exp(-(eta * dist) ** 2) / dist
            if i == j:
                phi = np.where(zero, 0.0, phi)
                dphi = np.where(zero, 0.0, dphi)
            e_real += 0.5 * z[i] * z[j] * np.sum(phi)
            # d|d|/dR_i = d/|d|, d|d|/dR_j = -d/|d|; (ddist/deps_ab = d_a d_b/|d|)
            fvec = z[i] * z[j] * 0.5 * (dphi / dist)[:, None] * d
            dR[i] += np.sum(fvec, axis=0)
            dR[j] -= np.sum(fvec, axis=0)
            deps += 0.5 * z[i] * z[j] * np.einsum("t,ta,tb->ab", dphi / dist, d, d)
    g2s = np.where(keep, g2, 1.0)
    ex = np.where(keep, np.exp(-g2s / (4.0 * eta ** 2)), 0.0)
    phase = np.exp(-1j * (g @ r.T))                         # (nG, nat)
    sf = np.sum(z[None, :] * phase, axis=-1)
    s2 = (sf * np.conj(sf)).real
    pref = 2.0 * np.pi / omega
    e_recip = pref * np.sum(ex / g2s * s2)
    # d|S|^2/dR_i = 2 Re[conj(S) z_i (-i G) e^{-iG.R_i}]
    w = ex / g2s
    for i in range(nat):
        dS = (np.conj(sf) * z[i] * (-1j) * phase[:, i]).real  # per G, times G_a
        dR[i] += pref * np.sum((2.0 * w * dS)[:, None] * g, axis=0)
    coef = np.where(keep, ex * (1.0 / (4.0 * eta ** 2 * g2s) + 1.0 / g2s ** 2) * 2.0, 0.0)
    deps += -e_recip * np.eye(3) + pref * np.einsum("g,ga,gb->ab", coef * s2, g, g)
    e_bg = -(np.pi / (2.0 * omega * eta ** 2)) * np.sum(z) ** 2
    deps += -e_bg * np.eye(3)
    return dR, deps


# --- occupations (occupation.py:25-72) -------------------------------------

def _sigmoid(x):
    return np.where(x >= 0, 1.0 / (1.0 + np.exp(-np.abs(x))),
                    np.exp(-np.abs(x)) / (1.0 + np.exp(-np.abs(x))))


def fermi(e, mu, sigma):
    return _sigmoid((mu - e) / sigma)


def occupations(eig, weights, nelec, sigma, spin_degeneracy=2.0, iters=80):
    """Fermi-Dirac with mu by 80 bisection steps; integer filling below 1e-6."""
    eig = np.asarray(eig, dtype=float)
    if sigma < 1e-6:
        return _integer_occupation(eig, weights, nelec, spin_degeneracy), 0.0
    lo = float(np.min(eig)) - 30.0 * sigma - 1.0
    hi = float(np.max(eig)) + 30.0 * sigma + 1.0
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        n = np.sum(weights[:, None] * fermi(eig, mid, sigma)) * spin_degeneracy
        if n > nelec:
            hi = mid
        else:
            lo = mid
    mu = 0.5 * (lo + hi)
    return fermi(eig, mu, sigma), mu


def _integer_occupation(eig, weights, nelec, spin_degeneracy):
    neff = nelec / spin_degeneracy
    flat_e = eig.reshape(-1)
    flat_w = np.broadcast_to(weights[:, None], eig.shape).reshape(-1)
    order = np.argsort(flat_e, kind="stable")
    cum = np.cumsum(flat_w[order])
    filled = cum <= neff + 1e-12
    last = int(np.argmax(cum > neff - 1e-12))
    frac = np.clip((neff - (cum[last] - flat_w[order][last])) / flat_w[order][last], 0.0, 1.0)
    vals = np.where(filled, 1.0, 0.0)
    vals[last] = vals[last] if filled[last] else frac
    out = np.zeros_like(flat_w)
    out[order] = vals
    return out.reshape(eig.shape)


def entropy(occ, weights):
    f = np.clip(occ, 1e-14, 1.0 - 1e-14)
    s = -(f * np.log(f) + (1.0 - f) * np.log(1.0 - f))
    return float(np.sum(weights[:, None] * s))


# ----------------------------------------------------------------------------
# Hamiltonian / Hpsi / SCF   (scf.py:36-92, 171-282; hpsi.py:18-50)
# ----------------------------------------------------------------------------

@dataclass
class GeometryCache:
    v_loc_r: np.ndarray
    proj: np.ndarray
    dion: np.ndarray


def build_geometry_cache(static, lattice, frac):
    """geometry_cache.py:32-39."""
    return GeometryCache(v_loc_r=local_potential_r(static, lattice, frac),
                         proj=projectors(static, lattice, frac),
                         dion=dion_full(static.psp, static.natom))


def kinetic_diag(basis, lattice, kpt):
    kg = gvectors(basis.miller, lattice, kpt)
    return 0.5 * np.sum(kg * kg, axis=-1)


def vmat_from_real(basis, v_r):
    """<G|V|G'> = fft(V)[(m_G - m_G') mod N]/N (scf.py:36-46)."""
    n1, n2, n3 = basis.fft_shape
    vg = np.fft.fftn(np.asarray(v_r).reshape(n1, n2, n3)) / basis.nfft
    m = basis.miller.astype(np.int64)
    d = m[:, None, :] - m[None, :, :]
    idx = (np.mod(d[..., 0], n1) * n2 + np.mod(d[..., 1], n2)) * n3 + np.mod(d[..., 2], n3)
    return vg.reshape(-1)[idx]


def effective_potential(static, lattice, rho_r, cache):
    """v_loc + v_H + v_xc (scf.py:81-92)."""
    v_h = hartree_potential_r(static.basis, lattice, rho_r)
    v_xc = xc_potential_point(rho_r)
    return cache.v_loc_r + v_h + v_xc, (cache.v_loc_r, v_h, v_xc)


def hamiltonian(static, lattice, v_r, cache):
    """Dense H = T + V + V_NL, hermitised (scf.py:54-78)."""
    vm = vmat_from_real(static.basis, v_r)
    hs = []
    for ik, k in enumerate(static.kpts):
        t = kinetic_diag(static.basis, lattice, k)
        vnl = np.einsum("pg,pq,qh->gh", cache.proj[ik], cache.dion, np.conj(cache.proj[ik]))
        h = np.diag(t) + vm + vnl
        hs.append(0.5 * (h + np.conj(h.T)))
    return np.stack(hs, axis=0)


def hpsi(static, lattice, psi, v_r, cache):
    """Matrix-free (T + V(r) + V_NL) psi (hpsi.py:18-50)."""
    basis = static.basis
    t = np.stack([psi[ik] * kinetic_diag(basis, lattice, k) for ik, k in enumerate(static.kpts)])
    v = real_to_psi(basis, lattice, psi_to_real(basis, lattice, psi) * v_r[None, None, :])
    return t + v + vnl_apply(cache.proj, cache.dion, psi)


def eigh_lowest(H, nband):
    """solver/eigh.py:30-41."""
    w, v = np.linalg.eigh(H)
    return w[..., :nband], np.swapaxes(v[..., :, :nband], -1, -2)


def scf_map(static, lattice, rho_r, cache):
    """n -> H[n] -> eigh -> occ -> n' (scf.py:171-183)."""
    v_r, _ = effective_potential(static, lattice, rho_r, cache)
    eig, vec = eigh_lowest(hamiltonian(static, lattice, v_r, cache), static.nband)
    occ, _ = occupations(eig, static.kweights, static.nelec, static.sigma, static.spin_degeneracy)
    return density_from_psi(static.basis, lattice, vec, occ, static.kweights, static.spin_degeneracy)


def density_residual(basis, lattice, rho_new, rho_old, nelec):
    """sum |drho| Omega/N/N_e (scf.py:226-229)."""
    return float(np.sum(np.abs(rho_new - rho_old)) * volume(lattice) / basis.nfft / nelec)


def initial_density(static, lattice):
    return np.full(static.basis.nfft, static.nelec / volume(lattice))


def q2_grid(basis, lattice):
    """|G|^2 on every box point, indices folded to [-n/2, n/2) (solver/scf.py:202-212)."""
    ax = [np.where(np.arange(n) < n // 2, np.arange(n), np.arange(n) - n) for n in basis.fft_shape]
    mm = np.stack(np.meshgrid(*ax, indexing="ij"), -1).astype(np.float64)
    g = mm @ reciprocal(lattice)
    return np.sum(g * g, axis=-1).reshape(-1)


def kerker_filter(basis, lattice, x, alpha, gg0):
    """alpha * K x, K = q^2/(q^2 + gg0) in G space, 0 at q = 0 (solver/scf.py:215-223)."""
    shape = tuple(basis.fft_shape)
    q2 = q2_grid(basis, lattice)
    filt = np.where(q2 > 1e-12, q2 / (q2 + gg0), 0.0)
    dg = np.fft.fftn(np.asarray(x).reshape(shape)).reshape(-1) * filt
    return alpha * np.fft.ifftn(dg.reshape(shape)).real.reshape(-1)


def kerker_mix(basis, lattice, rho_in, rho_out, alpha=0.5, gg0=1.0):
    """rho_in + alpha K (rho_out - rho_in) (solver/scf.py:215-223)."""
    return rho_in + kerker_filter(basis, lattice, rho_out - rho_in, alpha, gg0)


class DIISMixer:
    """Pulay/DIIS, history m = 8, restart on non-finite (mixer.py:23-82)."""

    def __init__(self, m=8, beta=0.5):
        self.m, self.beta = int(m), float(beta)
        self.rins, self.routs = [], []

    def reset(self):
        self.rins.clear()
        self.routs.clear()

    def __call__(self, rho_in, rho_out):
        self.rins.append(rho_in)
        self.routs.append(rho_out)
        if len(self.rins) > self.m:
            self.rins.pop(0)
            self.routs.pop(0)
        if len(self.rins) == 1:
            return rho_in + self.beta * (rho_out - rho_in)
        n = len(self.rins)
        rins, routs = np.stack(self.rins), np.stack(self.routs)
        res = routs - rins
        B = np.zeros((n + 1, n + 1))
        B[:n, :n] = res @ res.T
        B[:n, n] = -1.0
        B[n, :n] = -1.0
        B += np.eye(n + 1) * 1e-12
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        c = np.nan_to_num(np.linalg.solve(B, rhs)[:n], nan=0.0, posinf=0.0, neginf=0.0)
        new = np.einsum("i,ij->j", c, rins + self.beta * res)
        if not np.all(np.isfinite(new)):
            self.reset()
            return rho_in + self.beta * (rho_out - rho_in)
        return new


def solve_scf(system, tol=1e-10, max_iter=200, beta=0.5, rho0=None, verbose=False):
    """DIIS SCF + 4 polish steps + final eigh (scf.py:239-282)."""
    static, lat, frac = system.static, system.lattice, system.frac
    basis = static.basis
    cache = build_geometry_cache(static, lat, frac)
    rho = initial_density(static, lat) if rho0 is None else rho0
    mix = DIISMixer(m=8, beta=beta)
    prev, res, it = 1e9, 1.0, 0
    for it in range(1, max_iter + 1):
        rho_out = scf_map(static, lat, rho, cache)
        res = density_residual(basis, lat, rho_out, rho, static.nelec)
        if res > prev * 1.5:
            mix.reset()
        prev = res
        rho = mix(rho, rho_out)
        if verbose:
            print(f"  scf {it:3d} drho={res:.3e}")
        if res < tol:
            break
    for _ in range(4):
        rho_new = scf_map(static, lat, rho, cache)
        res = density_residual(basis, lat, rho_new, rho, static.nelec)
        rho = rho_new
        if res < 1e-14:
            break
    v_r, _ = effective_potential(static, lat, rho, cache)
    eig, vec = eigh_lowest(hamiltonian(static, lat, v_r, cache), static.nband)
    occ, mu = occupations(eig, static.kweights, static.nelec, static.sigma, static.spin_degeneracy)
    return SCFState(psi=vec, eig=eig, occ=occ, mu=mu, rho_r=rho, n_iter=it, residual=res)


# ----------------------------------------------------------------------------
# Energies   (observables/energy.py:22-169)
# ----------------------------------------------------------------------------
ALL_TAGS = ("kinetic", "local", "hartree", "exchange", "correlation", "nonlocal", "ewald")


def _kinetic_energy(static, lattice, state):
    total = 0.0
    for ik, k in enumerate(static.kpts):
        t = kinetic_diag(static.basis, lattice, k)
        w = static.kweights[ik] * state.occ[ik] * static.spin_degeneracy
        total += float(np.sum(w * np.sum(np.abs(state.psi[ik]) ** 2 * t[None, :], axis=-1)))
    return total


def _expect_potential(static, lattice, psi, occ, v_r):
    """sum w f g_s <psi|V|psi> through the dense matrix (energy.py:115-131)."""
    vm = vmat_from_real(static.basis, v_r)
    e = 0.0
    for ik in range(psi.shape[0]):
        hp = np.einsum("mn,bn->bm", vm, psi[ik])
        e += static.kweights[ik] * float(np.sum(occ[ik] * static.spin_degeneracy *
                                                np.sum(np.conj(psi[ik]) * hp, axis=-1).real))
    return e


def energy_terms(system, state, active=ALL_TAGS):
    """Seven tagged terms (energy.py:36-71)."""
    static, lat, frac = system.static, system.lattice, system.frac
    basis = static.basis
    out = {}
    if "kinetic" in active:
        out["kinetic"] = _kinetic_energy(static, lat, state)
    if "local" in active:
        out["local"] = _expect_potential(static, lat, state.psi, state.occ,
                                         local_potential_r(static, lat, frac))
    if "hartree" in active:
        out["hartree"] = hartree_energy(basis, lat, state.rho_r)
    if "exchange" in active:
        out["exchange"] = exchange_energy_lda(basis, lat, state.rho_r)
    if "correlation" in active:
        out["correlation"] = correlation_energy_lda(basis, lat, state.rho_r)
    if "nonlocal" in active:
        out["nonlocal"] = nonlocal_energy(projectors(static, lat, frac),
                                          dion_full(static.psp, static.natom), state.psi,
                                          state.occ, static.kweights, static.spin_degeneracy)
    if "ewald" in active:
        out["ewald"] = ewald_energy(lat, frac, np.full(static.natom, static.psp.zval),
                                    eta=static.eta_ewald)
    return out


def total_energy(system, state, active=ALL_TAGS):
    return float(sum(energy_terms(system, state, active).values()))


def energy_variational(system, state):
    """E = sum f<psi|H|psi> - E_H + E_xc - <psi|V_xc|psi> + E_II (energy.py:134-153)."""
    static, lat, frac = system.static, system.lattice, system.frac
    basis = static.basis
    cache = build_geometry_cache(static, lat, frac)
    v_r, (_, _, v_xc) = effective_potential(static, lat, state.rho_r, cache)
    H = hamiltonian(static, lat, v_r, cache)
    e_band = 0.0
    for ik in range(state.psi.shape[0]):
        hp = np.einsum("mn,bn->bm", H[ik], state.psi[ik])
        e_band += static.kweights[ik] * float(np.sum(
            state.occ[ik] * static.spin_degeneracy * np.sum(np.conj(state.psi[ik]) * hp, axis=-1).real))
    e_h = hartree_energy(basis, lat, state.rho_r)
    e_xc = xc_energy_lda(basis, lat, state.rho_r)
    e_dc = _expect_potential(static, lat, state.psi, state.occ, v_xc)
    e_ii = ewald_energy(lat, frac, np.full(static.natom, static.psp.zval), eta=static.eta_ewald)
    return e_band - e_h + e_xc - e_dc + e_ii


def mermin_free_energy(system, state):
    """F = E_var - sigma g_s S (energy.py:156-169)."""
    s = entropy(state.occ, system.static.kweights)
    return energy_variational(system, state) - system.static.sigma * system.static.spin_degeneracy * s


# ----------------------------------------------------------------------------
# Envelope gradients (api.py:94-118): psi and f frozen, rho = rho(geo, psi)
# ----------------------------------------------------------------------------

def envelope_gradients(system, state):
    """dF/dR (nat,3) and dF/deps (3,3) of the Mermin free energy with psi, f
    frozen and rho recomputed from psi at the current geometry (the reference's
    ``make_energy(mode="envelope")`` backward, api.py:106-113), hand-derived.

    With rho = rho(geo, psi) the variational form reduces to
    E_kin + E_NL + E_loc + E_H + E_xc + E_II - sigma g_s S, and every term is
    differentiated analytically here (cross-checked by central FD in tests).
    """
    static, lat, frac = system.static, system.lattice, system.frac
    basis, psp = static.basis, static.psp
    omega = volume(lat)
    nat = static.natom
    gs = static.spin_degeneracy
    psi, occ = state.psi, state.occ
    R = positions(lat, frac)
    rho = density_from_psi(basis, lat, psi, occ, static.kweights, gs)
    dR = np.zeros((nat, 3))
    deps = np.zeros((3, 3))
    eye = np.eye(3)

    # kinetic: d|k+G|^2/deps_ab = -2 (k+G)_a G_b  (k fixed cartesian, system.py:62)
    for ik, k in enumerate(static.kpts):
        g = gvectors(basis.miller, lat)
        kg = g + k[None, :]
        wf = static.kweights[ik] * occ[ik] * gs
        p2 = np.einsum("b,bg->g", wf, np.abs(psi[ik]) ** 2)
        deps += -np.einsum("g,ga,gb->ab", p2, kg, g)

    # Hartree (rho ~ 1/Omega): -E_H delta + 4 pi Omega sum |n|^2 G_a G_b / G^4
    ng = density_g(basis, rho)
    g = gvectors(basis.miller, lat)
    q2 = np.sum(g * g, axis=-1)
    m = q2 > 1e-14
    e_h = hartree_energy(basis, lat, rho)
    deps += -e_h * eye + FOUR_PI * omega * np.einsum(
        "g,ga,gb->ab", np.where(m, np.abs(ng) ** 2 / np.where(m, q2, 1.0) ** 2, 0.0), g, g)

    # XC: delta_ab (E_xc - (Omega/N) sum v_xc rho)
    e_xc = xc_energy_lda(basis, lat, rho)
    vxc = xc_potential_point(rho)
    deps += (e_xc - omega / basis.nfft * float(np.sum(vxc * rho))) * eye

    # local: E_loc = Re sum_G sum_I v~(|G|) e^{-iG.R_I} conj(n(G))  (rho shell)
    spec = np.fft.fftn(rho.reshape(basis.fft_shape)) / basis.nfft
    gr = gvectors(basis.miller_rho, lat)
    nr = grid_to_coeffs(basis.fft_shape, spec, basis.miller_rho)
    qr = safe_norm(gr)
    v0 = vloc_q(psp, qr)
    v1 = vloc_q_deriv(psp, qr)
    ph = np.exp(-1j * (gr @ R.T))                      # (nGr, nat)
    e_loc_terms = (v0[:, None] * ph * np.conj(nr)[:, None])
    e_loc = float(np.sum(e_loc_terms).real)
    for i in range(nat):
        dR[i] += np.sum(((-1j) * v0 * ph[:, i] * np.conj(nr))[:, None] * gr, axis=0).real
    sfc = np.sum(ph, axis=1) * np.conj(nr)              # S(G) conj(n(G))
    dq = np.where(qr > 0, -1.0 / np.where(qr > 0, qr, 1.0), 0.0)  # dq/deps_ab = -G_a G_b/q
    deps += -e_loc * eye + np.einsum("g,ga,gb->ab", (v1 * dq * sfc).real, gr, gr)

    # nonlocal: E_NL = sum w f g_s B^+ D B, beta_p ~ e^{-i(k+G).R_I}/sqrt(Omega)
    dion = dion_full(psp, nat)
    lm = psp.lm_table()
    nh = psp.nh
    e_nl = 0.0
    for ik, k in enumerate(static.kpts):
        g = gvectors(basis.miller, lat)
        kg = g + k[None, :]
        q = safe_norm(kg)
        ylm = ylm_real(psp.lmax, kg)
        dylm = ylm_real_grad(psp.lmax, kg)
        bet = beta_q(psp, q)
        dbet = beta_q_deriv(psp, q)
        u = np.where(q[:, None] > 0, kg / np.where(q > 0, q, 1.0)[:, None], 0.0)
        phase = np.exp(-1j * (kg @ R.T))
        rows, grads = [], []
        for i in range(nat):
            for ib, l, mm in lm:
                c = l * l + mm
                hat = bet[ib] * ylm[:, c]
                # gradient of the phase-free part w.r.t. v = k+G
                ghat = (dbet[ib] * ylm[:, c])[:, None] * u + bet[ib][:, None] * dylm[:, c, :]
                rows.append(hat * phase[:, i])
                grads.append(ghat * phase[:, i][:, None])
        beta = np.stack(rows) / np.sqrt(omega)              # (P, nG)
        Q = np.stack(grads) / np.sqrt(omega)                # (P, nG, 3)
        B = np.conj(beta) @ psi[ik].T                        # (P, nb)
        DB = dion @ B
        wf = static.kweights[ik] * occ[ik] * gs              # (nb,)
        e_nl += float(np.sum(wf * np.sum(np.conj(B) * DB, axis=0).real))
        # forces: dB_pa = sum_G i (k+G)_a conj(beta_p) psi
        dBR = np.einsum("pg,ga,bg->pab", np.conj(beta), 1j * kg, psi[ik])
        contrib = 2.0 * np.einsum("b,pab,pb->pa", wf, np.conj(dBR), DB).real   # (P,3)
        for i in range(nat):
            dR[i] += np.sum(contrib[i * nh:(i + 1) * nh], axis=0)
        # strain: d beta/deps_ab = -Q_a G_b - i k_b R_a beta - beta delta_ab/2
        X = np.einsum("pga,gb,ng->pabn", np.conj(Q), g, psi[ik])    # sum conj(Q_a) G_b psi
        Ratom = np.repeat(R, nh, axis=0)                            # (P,3)
        dBe = (-X + 1j * np.einsum("b,pa,pn->pabn", k, Ratom, B)
               - 0.5 * np.einsum("ab,pn->pabn", eye, B))
        deps += 2.0 * np.einsum("n,pabn,pn->ab", wf, np.conj(dBe), DB).real

    # Ewald
    dRe, depse = ewald_gradients(lat, frac, np.full(nat, psp.zval), eta=static.eta_ewald)
    dR += dRe
    deps += depse
    _ = e_nl
    return dR, deps


def forces_from_dR(dR):
    """F = -dE/dR (implicit.py:95-101 expressed in Cartesian form)."""
    return -np.asarray(dR)


def stress_from_deps(omega, deps):
    """sigma = -(1/Omega) sym(dE/deps) (api.py:145-146, implicit.py:104-110)."""
    g = np.asarray(deps)
    return -(0.5 * (g + g.T)) / omega


def energy_and_forces(system, **scf_kwargs):
    state = solve_scf(system, **scf_kwargs)
    e = mermin_free_energy(system, state)
    dR, _ = envelope_gradients(system, state)
    return e, forces_from_dR(dR), state


def stress(system, state=None, **scf_kwargs):
    state = solve_scf(system, **scf_kwargs) if state is None else state
    _, deps = envelope_gradients(system, state)
    return stress_from_deps(volume(system.lattice), deps)


def with_frac(system, frac):
    return replace(system, frac=np.asarray(frac, dtype=float))


def with_lattice(system, lattice):
    return replace(system, lattice=np.asarray(lattice, dtype=float))


# ----------------------------------------------------------------------------
# Explicit-table H psi for one k point (the CPU baseline of bench.py)
# ----------------------------------------------------------------------------

def hpsi_tables(fft_shape, miller, psi, kin, v_r, proj=None, dion=None, workers=None):
    """(T + V(r) + V_NL) psi with explicit tables, one k point (hpsi.py:18-50).

    psi (nb, nG); kin (nG,); v_r (N,); proj (P, nG); dion (P, P).  The FFT
    normalisations cancel to 1/N exactly as psi_to_real/real_to_psi give.
    ``workers`` selects scipy.fft with that many threads (None: numpy.fft).
    """
    import scipy.fft as sfft
    psi = np.asarray(psi)
    nb = psi.shape[0]
    n = int(np.prod(fft_shape))
    idx = flat_index(fft_shape, miller)
    grid = np.zeros((nb, n), dtype=psi.dtype)
    grid[:, idx] = psi
    grid = grid.reshape((nb,) + tuple(fft_shape))
    if workers:
        r = sfft.ifftn(grid, axes=(1, 2, 3), workers=workers, overwrite_x=True)
        r *= np.asarray(v_r).reshape(fft_shape)[None]
        spec = sfft.fftn(r, axes=(1, 2, 3), workers=workers, overwrite_x=True)
    else:
        r = np.fft.ifftn(grid, axes=(1, 2, 3)) * np.asarray(v_r).reshape(fft_shape)[None]
        spec = np.fft.fftn(r, axes=(1, 2, 3))
    out = spec.reshape(nb, n)[:, idx] + psi * np.asarray(kin)[None, :]
    if proj is not None:
        b = np.conj(proj) @ psi.T
        out = out + (proj.T @ (np.asarray(dion) @ b)).T
    return out


# ----------------------------------------------------------------------------
# Linear response and the fixed-point adjoint (physics/response.py:42-121,
# diff/implicit.py:32-110, observables/constraint.py:26-76)
# ----------------------------------------------------------------------------

def response_kernel(static, lattice, rho_r, dn):
    """K dn = v_H[dn] + f_xc(n) dn (response.py:70-76)."""
    return np.real(hartree_potential_r(static.basis, lattice, dn)) + xc_kernel_point(rho_r) * dn


def make_response(system, state, tol=1e-6, occupation_form="exact"):
    """(apply, chi0): dn -> (dF/dn) dn and dv -> density response, from the full
    dense eigensystem (response.py:42-121).  Pairs with |e_n - e_m| <= tol are
    dropped as in the reference.  Occupations: df = -f(1-f)/sigma (de - dmu) with
    one dmu for all k, the derivative of f = 1/(1 + exp((e - mu)/sigma))
    (occupation.py:18-20); the reference's response.py:104-107 writes +f(1-f)/sigma
    with a per-k dmu."""
    static, lat, frac = system.static, system.lattice, system.frac
    basis = static.basis
    cache = build_geometry_cache(static, lat, frac)
    v_r, _ = effective_potential(static, lat, state.rho_r, cache)
    hs = hamiltonian(static, lat, v_r, cache)
    nk, nb = state.psi.shape[0], static.nband
    eigs, vecs = [], []
    for ik in range(nk):
        w, v = np.linalg.eigh(hs[ik])
        c_occ = v[:, :nb]
        u, _, vh = np.linalg.svd(np.conj(c_occ).T @ state.psi[ik].T)
        v[:, :nb] = c_occ @ (u @ vh)
        eigs.append(w)
        vecs.append(v)
    f = np.asarray(state.occ, dtype=float)
    kw = np.asarray(static.kweights, dtype=float)
    g = static.spin_degeneracy
    fp = f * (1.0 - f) / static.sigma if static.sigma > 1e-6 else np.zeros_like(f)
    psi_r = psi_to_real(basis, lat, state.psi)

    def chi0(dv):
        dh = vmat_from_real(basis, dv)
        out = np.zeros(basis.nfft)
        de = np.zeros((nk, nb))
        for ik in range(nk):
            c, eps = vecs[ik], eigs[ik]
            m = np.conj(c).T @ dh @ c
            m = 0.5 * (m + np.conj(m).T)
            de[ik] = np.real(np.diag(m))[:nb]
            d = eps[None, :] - eps[:, None]
            off = np.abs(d) > tol
            coef = np.where(off, m / np.where(off, d, 1.0), 0.0)
            dc = (c @ coef)[:, :nb].T
            dpsi_r = psi_to_real(basis, lat, dc)
            out += kw[ik] * g * np.sum(f[ik][:, None] * 2.0 * np.real(np.conj(psi_r[ik]) * dpsi_r), axis=0)
        if static.sigma > 1e-6 and occupation_form == "reference":
            # the reference's own form (response.py:98-103): +f(1-f)/sigma and a shift per k
            dmu_k = np.sum(fp * de, axis=1, keepdims=True) / (np.sum(fp, axis=1, keepdims=True) + 1e-30)
            df = fp * (de - dmu_k)
            for ik in range(nk):
                out += kw[ik] * g * np.sum(df[ik][:, None] * np.abs(psi_r[ik]) ** 2, axis=0)
        elif static.sigma > 1e-6:
            wf = kw[:, None] * fp
            dmu = np.sum(wf * de) / (np.sum(wf) + 1e-300)
            df = -fp * (de - dmu)
            for ik in range(nk):
                out += kw[ik] * g * np.sum(df[ik][:, None] * np.abs(psi_r[ik]) ** 2, axis=0)
        return out

    def apply(dn):
        return chi0(response_kernel(static, lat, state.rho_r, dn))

    return apply, chi0


def delta_q(system, state, weight):
    """C = (Omega/N) sum_j w_j n_j (constraint.py:26-33)."""
    return volume(system.lattice) / system.static.basis.nfft * float(np.sum(weight * state.rho_r))


def make_gaussian_weight(basis, center, sigma=0.8, lattice=None):
    """Normalised Gaussian weight on the FFT grid (constraint.py:47-57)."""
    shape = tuple(basis.fft_shape)
    idx = np.stack(np.meshgrid(*(np.arange(n) for n in shape), indexing="ij"), -1).reshape(-1, 3)
    r = (idx / np.asarray(shape, dtype=float)) @ np.asarray(lattice, dtype=float)
    w = np.exp(-0.5 * np.sum((r - np.asarray(center)) ** 2, axis=-1) / sigma ** 2)
    return w / np.sum(w) * basis.nfft


def _geometry_fd(fn, lat, frac, h):
    """Central differences of a scalar fn(lattice, frac) in the Cartesian positions
    R = frac L and in the strain eps of strained(L, eps): (dR (nat, 3), deps (3, 3))."""
    pos = positions(lat, frac)
    dR = np.zeros_like(pos)
    for i in range(pos.shape[0]):
        for ax in range(3):
            vals = []
            for sgn in (1.0, -1.0):
                p = pos.copy()
                p[i, ax] += sgn * h
                vals.append(fn(lat, p @ np.linalg.inv(lat)))
            dR[i, ax] = (vals[0] - vals[1]) / (2 * h)
    deps = np.zeros((3, 3))
    for a_ in range(3):
        for b_ in range(3):
            vals = []
            for sgn in (1.0, -1.0):
                e = np.zeros((3, 3))
                e[a_, b_] = sgn * h
                vals.append(fn(strained(lat, e), frac))
            deps[a_, b_] = (vals[0] - vals[1]) / (2 * h)
    return dR, deps


def energy_dF_dn(system, state):
    """dF/dn of the Mermin free energy at fixed psi, f and geometry (the reference's
    g_n = jax.grad of the loss in rho_r, implicit.py:41).  The V_xc matrix elements of
    the band energy and of the double-counting term are the same function of n and
    cancel, leaving (Omega/N) (V_H[rho_psi] - V_H[n] + v_xc[n])."""
    static, lat = system.static, system.lattice
    basis = static.basis
    rho_psi = density_from_psi(basis, lat, state.psi, state.occ, static.kweights, static.spin_degeneracy)
    vh = lambda x: np.real(hartree_potential_r(basis, lat, x))  # noqa: E731
    return volume(lat) / basis.nfft * (vh(rho_psi) - vh(state.rho_r) + xc_potential_point(state.rho_r))


def implicit_grad_energy(system, state, h=1e-5):
    """The reference's make_energy(mode="adjoint") backward for the Mermin free energy
    (api.py:114-116 -> implicit.py:32-87): dense A = I - dF_map/dn, A^T lambda = dF/dn
    (energy_dF_dn), the state term dF/dtheta at fixed (psi, f, n) and lambda^T dF_map/dtheta
    at fixed n, both by central differences.  Returns (dF/dR (nat, 3), dF/deps (3, 3))."""
    static, lat, frac = system.static, system.lattice, system.frac
    nfft = static.basis.nfft
    apply, _ = make_response(system, state)
    jac = np.stack([apply(e) for e in np.eye(nfft)], axis=1)
    lam = np.linalg.solve((np.eye(nfft) - jac).T, energy_dF_dn(system, state))
    n_star = state.rho_r

    def f_state(lat_, frac_):
        return mermin_free_energy(System(lattice=lat_, frac=frac_, static=static), state)

    def lmap(lat_, frac_):
        return float(lam @ scf_map(static, lat_, n_star, build_geometry_cache(static, lat_, frac_)))

    dR1, de1 = _geometry_fd(f_state, lat, frac, h)
    dR2, de2 = _geometry_fd(lmap, lat, frac, h)
    return dR1 + dR2, de1 + de2


def implicit_grad_delta_q(system, state, weight, h=1e-5):
    """dC/dgeo for C = delta_q by the fixed-point adjoint (implicit.py:32-87):
    dense A = I - dF/dn, (A^T) lambda = dC/dn, and lambda^T dF/dtheta at fixed n by
    central differences of lambda . scf_map (the map alone, no SCF).
    Returns (dC/dR (nat, 3), dC/deps (3, 3), lambda)."""
    static, lat, frac = system.static, system.lattice, system.frac
    nfft = static.basis.nfft
    apply, _ = make_response(system, state)
    jac = np.stack([apply(e) for e in np.eye(nfft)], axis=1)
    a = np.eye(nfft) - jac
    gn = volume(lat) / nfft * np.asarray(weight, dtype=float)
    lam = np.linalg.solve(a.T, gn)
    n_star = state.rho_r

    def lmap(lat_, frac_):
        cache = build_geometry_cache(static, lat_, frac_)
        return float(lam @ scf_map(static, lat_, n_star, cache))

    pos = positions(lat, frac)
    dR = np.zeros_like(pos)
    for i in range(pos.shape[0]):
        for ax in range(3):
            vals = []
            for sgn in (1.0, -1.0):
                p = pos.copy()
                p[i, ax] += sgn * h
                vals.append(lmap(lat, p @ np.linalg.inv(lat)))
            dR[i, ax] = (vals[0] - vals[1]) / (2 * h)
    deps = np.zeros((3, 3))
    for a_ in range(3):
        for b_ in range(3):
            vals = []
            for sgn in (1.0, -1.0):
                e = np.zeros((3, 3))
                e[a_, b_] = sgn * h
                vals.append(lmap(strained(lat, e), frac))
            deps[a_, b_] = (vals[0] - vals[1]) / (2 * h)
    deps += delta_q(system, state, weight) * np.eye(3)      # d Omega / d eps at fixed n
    return dR, deps, lam
