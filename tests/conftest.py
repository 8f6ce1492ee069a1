"""Shared test setup.

* registers the ``gpu`` marker (tests that need a GB300 and the built
  libaddft_gb300.so; the CPU suite runs with ``-m "not gpu"``);
* puts the repo root (for ``oracle``) and ``ad-dft_gb300`` (for the
  ``addft_gb300`` package) on ``sys.path``;
* the fixture system is the reference's own (tests/conftest.py:26-34 there):
  6 Bohr cubic cell, frac (0,0,0)/(0.53,0.47,0.49), ecut 2 Ha, nband 2,
  density_factor 4, sigma 0.05 -> nG 27, box 9^3.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "ad-dft_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

LATTICE = np.eye(3) * 6.0
FRAC_DISTORTED = np.array([[0.0, 0.0, 0.0], [0.53, 0.47, 0.49]])
FRAC_SYMMETRIC = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device and the built libaddft_gb300.so")
    config.addinivalue_line("markers", "slow: long-running (multi-SCF finite differences)")


def oracle_system(frac=FRAC_DISTORTED, ecut=2.0, nband=2, factor=4.0, sigma=0.05, kmesh=None):
    from oracle import pw
    return pw.setup(LATTICE, frac, ecut=ecut, nband=nband, density_factor=factor, sigma=sigma, kmesh=kmesh)


@pytest.fixture(scope="session")
def osys():
    return oracle_system()


@pytest.fixture(scope="session")
def ostate(osys):
    from oracle import pw
    return pw.solve_scf(osys)


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
