"""The product path has no CPU fallback, checked on a host without a GPU: importing the package
without its CUDA library raises ImportError naming the build step, and every call that would launch
kernels (a plan, an SCF) raises instead of computing on the CPU.  The oracle is never reached."""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")


def test_import_without_the_cuda_library_raises():
    env = dict(os.environ, ADDFT_GB300_LIB="/nonexistent/libaddft_gb300.so", PYTHONPATH=str(ROOT / "ad-dft_gb300"))
    r = subprocess.run([sys.executable, "-c", "import addft_gb300"], env=env, capture_output=True, text=True)
    assert r.returncode != 0
    assert "ImportError" in r.stderr and "is not built" in r.stderr


def test_calls_that_launch_kernels_raise_without_a_gpu():
    import addft_gb300 as ad
    from addft_gb300 import ops
    with pytest.raises(RuntimeError, match="CUDA device"):
        ops.Plan((9, 9, 9), np.zeros((1, 3), dtype=np.int32))
    s = ad.setup(np.eye(3) * 6.0, [[0, 0, 0], [0.53, 0.47, 0.49]], ecut=2.0, nband=2, density_factor=4.0)
    with pytest.raises(RuntimeError):
        ad.scf(s)


def test_no_product_module_imports_the_oracle():
    """The oracle is the checker only: nothing in the package (Python or CUDA sources) imports it."""
    pkg = ROOT / "ad-dft_gb300"
    for f in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")):
        text = f.read_text()
        assert "import oracle" not in text and "from oracle" not in text and "oracle/" not in text, f
