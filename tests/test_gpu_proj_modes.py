"""Every kernel of the FP32 projector contractions against the FP64 kernels.

The kernel is chosen once per process (ADDFT_BECP_TC / ADDFT_APPLY_TC: 0 register-
tiled FP32 FMA, 1 split-TF32 mma.sync, 2 generic SIMT, 3 split-TF32 tcgen05 with a
tensor-memory accumulator), so each choice runs in a child process.  Shapes cover
partial band / projector / G tiles, several k points and the 256-projector chunking
of the tcgen05 apply.  Tolerance 1e-5 relative (the reference's FP32 bar is 2e-3,
tests/test_hpsi.py:53-72); the tcgen05 kernels must also report no expired waits.
"""

from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu
if not gpu_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import json, sys
sys.path[:0] = [%r, %r]
import torch
from addft_gb300 import ops
from addft_gb300._lib import LIB
g = torch.Generator(device="cuda").manual_seed(9)
def rnd(*s):
    return torch.complex(torch.randn(*s, generator=g, device="cuda"), torch.randn(*s, generator=g, device="cuda"))
out = {}
for (nk, nb, P, nG) in [(1, 64, 32, 4099), (1, 3, 4, 517), (2, 100, 40, 3001), (3, 17, 33, 64), (1, 160, 256, 2000)]:
    proj, psi = rnd(nk, P, nG), rnd(nk, nb, nG)
    b = ops.becp(proj, psi)
    bref = ops.becp(proj.to(torch.complex128), psi.to(torch.complex128))
    d = torch.randn(P, P, generator=g, device="cuda")
    d = 0.5 * (d + d.T)
    h0 = rnd(nk, nb, nG)
    h = h0.clone()
    ops.vnl_apply(proj, d, b, h)
    h64 = h0.to(torch.complex128)
    ops.vnl_apply(proj.to(torch.complex128), d.double(), b.to(torch.complex128), h64)
    torch.cuda.synchronize()
    key = "%%dx%%dx%%dx%%d" %% (nk, nb, P, nG)
    out[key] = [float((b.to(torch.complex128) - bref).abs().max() / bref.abs().max()),
                float((h.to(torch.complex128) - h64).abs().max() / (h64 - h0.to(torch.complex128)).abs().max())]
out["status"] = int(LIB.addft_tc05_status())
print("RESULT " + json.dumps(out))
"""


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_projector_kernels_match_fp64(mode):
    env = dict(os.environ, ADDFT_BECP_TC=str(mode), ADDFT_APPLY_TC=str(mode))
    code = CHILD % (str(ROOT), str(ROOT / "ad-dft_gb300"))
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    line = [ln for ln in res.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    out = json.loads(line[len("RESULT "):])
    assert out.pop("status") == 0
    for key, (eb, ea) in out.items():
        assert eb < 1e-5 and ea < 1e-5, (mode, key, eb, ea)
