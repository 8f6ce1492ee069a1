"""The C ABI from C: include/addft_gb300.h compiles as plain C99 (-Wall -Werror) and a C
program linked against libaddft_gb300.so calls entry points whose argument checks run
before any CUDA call (no GPU needed)."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "ad-dft_gb300" / "addft_gb300" / "libaddft_gb300.so"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_header_compiles_as_c99_and_links(tmp_path):
    if not LIB.exists():
        pytest.skip("library not built")
    exe = tmp_path / "abi_check"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "c" / "abi_check.c"), "-o", str(exe), str(LIB), f"-Wl,-rpath,{LIB.parent}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "abi_check ok" in run.stdout
