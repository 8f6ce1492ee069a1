"""The oracle's checks fail on planted mistakes (the reference's tests/test_harness_catches_bugs.py).

Known bug classes are planted in the oracle, on the CPU, with monkeypatch; the check that guards
each class must then raise.  A check that still passed with the mistake planted would be too weak to
pin the CUDA path against.  The reference's three classes:

* v_xc with the wrong weight (0.5 v_xc)      -> v_xc against d(n eps_xc)/dn by central differences;
* D in the per-atom-pair layout               -> V_NL Hermiticity and D's block-diagonal layout;
* k points in the wrong unit (2 pi k_frac)    -> the 2x2x2 mesh's largest |k| component;

and one more, the layout mistake a transform kernel most often makes:

* the real-space grid transposed (flat index (i3 n2 + i2) n1 + i1)
                                              -> H psi and density against the values the
                                                 reference's own code produced (microbench 15^3).
Each unplanted check passes in its own test module; here only the planted runs are made.
"""

from __future__ import annotations

import numpy as np
import pytest

import test_oracle_pins as pins   # modules, not their test functions: pytest collects those only there
import test_reference_fixtures as fixtures
from oracle import pw


def test_harness_catches_wrong_xc_weight(monkeypatch):
    good = pw.xc_potential_point
    monkeypatch.setattr(pw, "xc_potential_point", lambda n: 0.5 * good(n))
    with pytest.raises(AssertionError):
        pins.test_xc_potential_and_kernel_are_derivatives()


def test_harness_catches_per_atom_pair_dion_layout(monkeypatch, osys, ostate):
    good = pw.dion_full

    def pair_layout(psp, natom):
        d0 = good(psp, natom)
        nh = d0.shape[0] // natom
        d = np.zeros((natom, natom, nh, nh), dtype=d0.dtype)
        for i in range(natom):
            d[i, i] = d0[i * nh:(i + 1) * nh, i * nh:(i + 1) * nh]
        return d.reshape(natom * nh, natom * nh)   # (atom, atom, h, h) read as (atom h, atom h)

    monkeypatch.setattr(pw, "dion_full", pair_layout)
    with pytest.raises(AssertionError):
        pins.test_nonlocal_is_hermitian_and_dion_block_diagonal(osys, ostate)


def test_harness_catches_wrong_kpoint_unit(monkeypatch):
    monkeypatch.setattr(pw.KMesh, "cartesian", lambda self, lattice: 2.0 * np.pi * self.kfrac)
    with pytest.raises(AssertionError):
        pins.test_box_rule_and_kweights()


def test_harness_catches_transposed_real_space_grid(monkeypatch):
    def transposed(shape, miller):
        n1, n2, n3 = shape
        m = np.asarray(miller)
        return ((np.mod(m[:, 2], n3) * n2 + np.mod(m[:, 1], n2)) * n1 + np.mod(m[:, 0], n1)).astype(np.int64)

    monkeypatch.setattr(pw, "flat_index", transposed)
    with pytest.raises(AssertionError):
        fixtures.test_oracle_hpsi_and_density_match_reference_microbench("15")
