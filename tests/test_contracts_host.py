"""The reference's contract tests (tests/test_contracts.py) on this package's host side, no GPU:
the single Ry / Ha unit bridge, 2,3,5-smooth FFT lengths (7 excluded, after ABACUS), the box rule
"2 n + 1, then up to the next smooth length", the frozen shell with G = 0 and its reported margin,
and k weights that sum to one.  The energy-decomposition tags are switched on the GPU
(tests/test_gpu_scf.py)."""

from __future__ import annotations

import numpy as np

import addft_gb300 as ad
from addft_gb300 import geometry as G
from addft_gb300 import units


def test_unit_bridge():
    assert units.RY_TO_HA == 0.5
    assert abs(units.HA_TO_EV - 27.211386245988) < 1e-9
    assert abs(units.ry_to_ha(30.0) - 15.0) < 1e-12 and abs(units.ha_to_ry(15.0) - 30.0) < 1e-12
    assert ad.units is units


def test_smooth_numbers_only_235():
    assert G.is_smooth235(12) and G.is_smooth235(15) and G.is_smooth235(27)
    assert not G.is_smooth235(7) and not G.is_smooth235(14) and not G.is_smooth235(49)
    assert (G.smooth_up(7), G.smooth_up(11), G.smooth_up(13)) == (8, 12, 15)
    smooth = [n for n in range(1, 200) if G.is_smooth235(n)]
    assert all(G.smooth_up(n) == min(m for m in smooth if m >= n) for n in range(1, 180))


def test_fft_box_is_odd_then_smooth():
    lat = np.eye(3) * 6.0
    shape = G.fft_shape(lat, 2.0, density_factor=4.0)
    assert isinstance(shape, tuple) and all(G.is_smooth235(n) for n in shape)
    # 2 m + 1 points on each axis, m = ceil(|G|max |a_i| / 2 pi) the density sphere's extent along
    # reciprocal axis i, rounded up to the next smooth length; the box then holds the density shell
    m = np.ceil(np.sqrt(2.0 * 2.0 * 4.0) * np.linalg.norm(lat, axis=1) / (2 * np.pi)).astype(int)
    assert shape == tuple(G.smooth_up(2 * int(x) + 1) for x in m)
    rho = G.build_miller(lat, 2.0 * 4.0)
    assert all(2 * int(np.max(np.abs(rho[:, a]))) + 1 <= n for a, n in enumerate(shape))


def test_shell_is_frozen_and_margin_reported():
    lat = np.eye(3) * 6.0
    basis = G.make_basis(lat, 2.0)
    assert basis.miller.dtype == np.int32
    assert np.any(np.all(basis.miller == 0, axis=1))
    m = G.shell_margin(basis, lat)
    assert 0.0 < m < 1.0
    assert np.array_equal(G.make_basis(lat, 2.0).miller, basis.miller)   # deterministic order


def test_kmesh_weights_sum_to_one():
    for km in (G.gamma(), G.monkhorst_pack((2, 2, 2)), G.monkhorst_pack((3, 1, 1), (0.5, 0, 0))):
        assert G.check_weights(km) < 1e-14


def test_synthetic_pseudopotential_has_its_m_channels():
    """l = (0, 1) gives 1 + 3 projector channels per atom (tests/test_ylm.py:41-52)."""
    psp = ad.synthetic()
    assert psp.proj_l == (0, 1) and psp.nh == 4
    from addft_gb300.psp import dion_full
    assert dion_full(psp, 2).shape == (8, 8)
