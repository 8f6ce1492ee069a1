"""CPU-only checks of the C ABI library and the host-side setup logic.

No kernel is launched here: the library is loaded, every symbol declared in
include/addft_gb300.h must be exported, argument validation that runs before
any CUDA call is exercised, and the host basis builder must reproduce the
oracle's (= the reference's) Miller ordering and FFT boxes bit for bit.
"""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "addft_gb300.h"
LIB = ROOT / "ad-dft_gb300" / "addft_gb300" / "libaddft_gb300.so"


@pytest.fixture(scope="module")
def lib():
    if not LIB.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("addft_gb300_build", LIB.parent / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    return C.CDLL(str(LIB))


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(addft_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_hot_path():
    syms = declared_symbols()
    for s in ("addft_hpsi", "addft_density", "addft_xc_lda", "addft_hartree", "addft_becp",
              "addft_vnl_apply", "addft_projectors", "addft_local_potential", "addft_ewald",
              "addft_nonlocal_gradients", "addft_density_gradients", "addft_kinetic_stress",
              "addft_occupations", "addft_psi_to_real", "addft_real_to_psi"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_every_declared_symbol(lib):
    from addft_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.EXPORTED)


def test_status_strings_and_version(lib):
    lib.addft_status_string.restype = C.c_char_p
    assert lib.addft_status_string(0) == b"ok"
    assert lib.addft_status_string(1) == b"invalid argument"
    assert lib.addft_status_string(5) == b"unsupported"
    assert lib.addft_version() >= 1


def test_plan_validation_runs_before_any_cuda_call(lib):
    lib.addft_plan_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.POINTER(C.c_int32)]
    lib.addft_last_error.restype = C.c_char_p
    h = C.c_void_p()
    m = np.array([[0, 0, 0], [9, 0, 0]], dtype=np.int32)       # aliases in a 9^3 box
    st = lib.addft_plan_create(C.byref(h), 9, 9, 9, 2, m.ctypes.data_as(C.POINTER(C.c_int32)))
    assert st == 1 and b"aliases" in lib.addft_last_error()
    st = lib.addft_plan_create(C.byref(h), 7, 9, 9, 2, m.ctypes.data_as(C.POINTER(C.c_int32)))
    assert st == 5 and b"smooth" in lib.addft_last_error()
    assert lib.addft_plan_create(C.byref(h), 9, 9, 9, 0, m.ctypes.data_as(C.POINTER(C.c_int32))) == 1


@pytest.mark.parametrize("lat,ecut,factor,kmesh", [
    (np.eye(3) * 6.0, 2.0, 4.0, None),
    (np.eye(3) * 6.0, 2.0, 2.0, None),
    (np.eye(3) * 6.0, 2.0, 4.0, (2, 2, 2)),
    (np.eye(3) * 10.26, 10.0, 4.0, None),
    (np.array([[0.0, 5.13, 5.13], [5.13, 0.0, 5.13], [5.13, 5.13, 0.0]]), 8.0, 4.0, (2, 2, 2)),
])
def test_host_basis_matches_oracle_bit_exact(lat, ecut, factor, kmesh):
    from addft_gb300 import geometry as G
    from oracle import pw
    km_p = G.monkhorst_pack(kmesh) if kmesh else G.gamma()
    km_o = pw.monkhorst_pack(kmesh) if kmesh else pw.gamma()
    bp = G.make_basis(lat, ecut, factor, kpts=km_p.cartesian(lat))
    bo = pw.make_basis(lat, ecut, factor, kpts=km_o.cartesian(lat))
    assert bp.fft_shape == bo.fft_shape
    assert np.array_equal(bp.miller, bo.miller)
    assert np.array_equal(bp.miller_rho, bo.miller_rho)


def test_dion_full_matches_oracle():
    from addft_gb300.psp import dion_full, synthetic
    from oracle import pw
    assert np.array_equal(dion_full(synthetic(), 3), pw.dion_full(pw.synthetic(), 3))


def test_psp_struct_and_rejections():
    import addft_gb300 as ad
    s = ad.synthetic().c_struct()
    assert s.nrad == 2 and list(s.l)[:2] == [0, 1] and abs(s.w[1] - 0.6) < 1e-15
    with pytest.raises(NotImplementedError):
        ad.synthetic(zval=(2.0, 4.0))
    with pytest.raises(NotImplementedError):
        ad.setup(np.eye(3) * 6, [[0, 0, 0], [0.5, 0.5, 0.5]], spec_idx=[0, 1])


def test_setup_without_gpu_builds_static():
    import addft_gb300 as ad
    s = ad.setup(np.eye(3) * 6.0, [[0, 0, 0], [0.53, 0.47, 0.49]], ecut=2.0, nband=2, density_factor=4.0)
    assert s.static.basis.nG == 27 and s.static.basis.fft_shape == (9, 9, 9)
    assert s.static.nelec == 4.0 and s.static.sigma == 0.05


def test_reference_shaped_and_host_entry_points_validate_before_any_cuda_call(lib):
    """The FFI-handler-shaped entry points and the host-buffer H psi reject bad arguments with
    ADDFT_INVALID_ARG (the handlers' ffi::Error::InvalidArgument) before touching the device."""
    from addft_gb300 import _lib as L
    LIB = L.LIB
    n = C.c_void_p(0)
    # XcLdaHandler: missing output / work
    assert LIB.addft_ffi_xc_lda(4, n, n, n, n, 0, n) == 1
    assert LIB.addft_ffi_xc_lda_work_bytes() >= 8 * 256
    # Scatter / Gather: negative sizes, empty grid
    assert LIB.addft_ffi_scatter(1, -1, 4, 8, n, n, n, n) == 1
    assert LIB.addft_ffi_gather(0, 1, 4, 0, n, n, n, n) == 1
    assert LIB.addft_ffi_check_index(3, 8, n, n, n) == 1
    # EighLowestHandler: "nband > nG" and bad sizes
    assert LIB.addft_ffi_eigh_lowest(1, 4, 5, n, n, n, n, 0, n) == 1
    assert b"nband" in LIB.addft_last_error()
    assert LIB.addft_ffi_eigh_lowest(1, 0, 0, n, n, n, n, 0, n) == 1
    # host-buffer H psi: no plan, no buffers
    assert LIB.addft_hpsi_host(n, 0, 1, 4, n, n, n, 0, n, n, n, 2, n, 0, n) == 1
    assert LIB.addft_hpsi_host_work_bytes(n, 0, 1, 4, 0, 2) == 0
    # empty batches are no-ops
    assert LIB.addft_ffi_scatter(1, 0, 4, 8, n, n, n, n) == 0
    assert LIB.addft_ffi_gather(1, 3, 0, 8, n, n, n, n) == 0


def _index_checks(m):
    m = np.asarray(m, dtype=np.int64)
    w = np.arange(1, m.shape[0] + 1, dtype=np.int64)
    return {"n": int(m.shape[0]), "wsum": [int(x) for x in (w[:, None] * m).sum(axis=0)],
            "sq": int(np.sum(m * m)), "head": m[:8].tolist(), "tail": m[-8:].tolist()}


def test_host_basis_and_kmesh_match_reference_code():
    """The host basis builder and Monkhorst-Pack meshes against the reference's own
    geometry/basis.py make_basis and geometry/kmesh.py (tests/golden/make_reference_fixtures.py):
    the Miller sets of the wavefunction and density shells in their frozen order (an order-
    weighted checksum, the sum of squares and both ends) and the FFT boxes exactly, the k
    points and weights to 1e-15."""
    import json
    from addft_gb300 import geometry as G
    fix = json.loads((ROOT / "tests" / "golden" / "ref_fixtures.json").read_text())["basis"]
    for name, c in fix.items():
        lat = np.asarray(c["lattice"])
        km = G.monkhorst_pack(tuple(c["kmesh"])) if c["kmesh"] else G.gamma()
        assert np.allclose(km.kfrac, c["kfrac"], rtol=0, atol=1e-15), name
        assert np.allclose(km.weights, c["kweights"], rtol=0, atol=1e-15), name
        b = G.make_basis(lat, c["ecut"], c["density_factor"], kpts=km.cartesian(lat))
        assert list(b.fft_shape) == c["fft_shape"], name
        assert _index_checks(b.miller) == c["miller"], name
        assert _index_checks(b.miller_rho) == c["miller_rho"], name
