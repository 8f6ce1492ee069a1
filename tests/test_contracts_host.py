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


def test_batch_autotuner_candidates_use_valid_tuning_keys_and_values():
    """Every launch shape the batch autotuner tries is a valid plan tuning (keys that
    addft_plan_set_tuning knows, values inside its ranges), so a tune() on the GPU never
    stops on a rejected candidate."""
    from addft_gb300.batch import default_candidates
    from addft_gb300.ops import Plan
    ranges = {"colfft": {0, 1, 2}, "plane2": {0, 1}, "xline2": {0, 1}, "xy_direct": {0, 1}, "plane_split": {0, 1}}
    cands = default_candidates()
    assert cands and len({tuple(sorted(c.items())) for c in cands}) == len(cands)   # no duplicates
    for c in cands:
        assert set(c) <= set(Plan.TUNING_KEYS), c
        for k, v in c.items():
            if k in ranges:
                assert v in ranges[k], (k, v)
            elif k in ("threads_plane", "threads_x", "threads_plane2"):
                assert 64 <= v <= 512 and v % 32 == 0, (k, v)
            elif k == "threads_xy":
                assert v == 0 or (64 <= v and v % 32 == 0), (k, v)
            elif k == "slab_mb":
                assert 1 <= v <= 1 << 20


def test_configuration_bases_have_the_reference_sizes():
    """The benchmark configurations' shells and boxes as the reference's own rules give them
    (basis.py:80-132): the fixture cell nG 27 in 9^3, Si8 at ecut 10 nG 1647 in 32^3, Si64 at ecut 15
    nG 23,847 in 75^3, and the eight-structure batch at ecut 8 (Gamma shells): Si2 283 / 24^3,
    Si4 585 / 24x24x30, Si8 1189 / 30^3, Si16 2355 / 30x30x60, Si32 4701 / 60x60x30."""
    for lat, ecut, nG, box in ((np.eye(3) * 6.0, 2.0, 27, (9, 9, 9)),
                               (np.eye(3) * 10.26, 10.0, 1647, (32, 32, 32)),
                               (np.eye(3) * 20.52, 15.0, 23847, (75, 75, 75))):
        b = G.make_basis(lat, ecut, 4.0)
        assert (b.nG, b.fft_shape) == (nG, box)
    from addft_gb300.batch import silicon_batch
    got = [(s.static.natom, s.static.basis.nG, s.static.basis.fft_shape)
           for s in silicon_batch(kmesh=None, sigma_disp=0.0)]
    assert got == [(2, 283, (24, 24, 24)), (4, 585, (24, 24, 30)), (8, 1189, (30, 30, 30)), (8, 1189, (30, 30, 30)),
                   (16, 2355, (30, 30, 60)), (16, 2355, (30, 30, 60)), (32, 4701, (60, 60, 30)),
                   (32, 4701, (60, 60, 30))]


def test_microbench_spheres_have_the_reference_sizes():
    """The H psi microbench's spheres of radius 0.45 n: 9^3 -> 257, 15^3 -> 1309, 48^3 -> 42,211,
    72^3 -> 142,609 points."""
    import bench
    assert [bench.sphere_miller(n).shape[0] for n in (9, 15, 48, 72)] == [257, 1309, 42211, 142609]
