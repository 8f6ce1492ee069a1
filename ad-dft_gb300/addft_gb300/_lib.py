"""ctypes binding of libaddft_gb300.so (the C ABI declared in include/addft_gb300.h).

This is the only way the package reaches the GPU kernels.  There is no CPU
fallback: importing this module raises if the shared library is missing, and
every call raises ``AddftError`` on a non-OK status.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_LIB_PATH = Path(os.environ.get("ADDFT_GB300_LIB", Path(__file__).resolve().parent / "libaddft_gb300.so"))

F32, F64 = 0, 1


class AddftError(RuntimeError):
    pass


class Psp(C.Structure):
    """addft_psp: KB pseudopotential of one species (analytic or tabulated)."""
    _fields_ = [("nrad", C.c_int), ("l", C.c_int * 4), ("w", C.c_double * 4), ("b", C.c_double * 4),
                ("vloc_amp", C.c_double), ("vloc_sigma", C.c_double), ("kind", C.c_int), ("nq", C.c_int),
                ("dq", C.c_double), ("tab", C.c_void_p), ("vloc_g0", C.c_double), ("zval", C.c_double)]


def _load():
    if not _LIB_PATH.exists():
        raise ImportError(
            f"{_LIB_PATH} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the GB300 kernels have no CPU fallback)")
    lib = C.CDLL(str(_LIB_PATH))
    P, I, D, S, V = C.c_void_p, C.c_int, C.c_double, C.c_size_t, C.c_void_p
    DP = C.POINTER(C.c_double)
    sigs = {
        "addft_status_string": (C.c_char_p, [I]),
        "addft_last_error": (C.c_char_p, []),
        "addft_version": (I, []),
        "addft_launch_count": (C.c_ulonglong, []),
        "addft_plan_create": (I, [C.POINTER(P), I, I, I, I, C.POINTER(C.c_int32)]),
        "addft_plan_destroy": (I, [P]),
        "addft_plan_info": (I, [P, C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
        "addft_plan_set_tuning": (I, [P, C.c_char_p, C.c_long]),
        "addft_plan_get_tuning": (I, [P, C.c_char_p, C.POINTER(C.c_long)]),
        "addft_work_bytes": (S, [P, I, I]),
        "addft_hpsi_work_bytes": (S, [P, I, I, I, I, I]),
        "addft_hartree_work_bytes": (S, [P]),
        "addft_local_potential_work_bytes": (S, [P]),
        "addft_density_gradients_work_bytes": (S, [P, P, I]),
        "addft_nonlocal_gradients_work_bytes": (S, [I, I, I, I, I, I]),
        "addft_ewald_work_bytes": (S, [I]),
        "addft_psi_to_real": (I, [P, I, I, D, V, V, V, S, V]),
        "addft_real_to_psi": (I, [P, I, I, D, V, V, V, S, V]),
        "addft_kinetic": (I, [P, I, DP, I, DP, V, V]),
        "addft_hpsi": (I, [P, I, I, I, V, V, V, I, V, V, V, V, S, V]),
        "addft_hpsi_noalloc": (I, [P, I, I, I, V, V, V, I, V, V, V, V]),
        "addft_hpsi_noalloc_max_scratch_bytes": (S, []),
        "addft_hpsi_host": (I, [P, I, I, I, V, V, V, I, V, V, V, I, V, S, V]),
        "addft_hpsi_host_work_bytes": (S, [P, I, I, I, I, I]),
        "addft_becp": (I, [I, I, I, I, I, V, V, V, V, S, V]),
        "addft_vnl_apply": (I, [I, I, I, I, I, V, V, V, V, V, S, V]),
        "addft_nonlocal_energy": (I, [I, I, I, I, V, V, V, V, V, S, V]),
        "addft_projectors": (I, [P, I, DP, D, I, DP, I, DP, C.POINTER(Psp), V, V]),
        "addft_density": (I, [P, I, I, I, D, V, V, V, V, S, V]),
        "addft_xc_lda": (I, [I, V, V, V, V, V, V, V, V, S, V]),
        "addft_xc_lda_vjp": (I, [I, V, V, V, V]),
        "addft_hartree": (I, [P, DP, D, V, V, V, V, S, V]),
        "addft_local_potential": (I, [P, DP, D, I, DP, C.POINTER(Psp), V, V, S, V]),
        "addft_ewald": (I, [DP, I, DP, DP, D, I, V, V, S, V]),
        "addft_occupations": (I, [I, I, V, V, D, D, D, I, V, V, V]),
        "addft_kerker": (I, [P, DP, V, D, D, V, V, S, V]),
        "addft_kerker_work_bytes": (S, [P]),
        "addft_zgemm_df": (I, [I, I, I, V, C.c_long, C.c_long, I, V, C.c_long, C.c_long, I, V, C.c_long, V, S, V]),
        "addft_zgemm_df_work_bytes": (S, [I, I, I]),
        "addft_peak_flops": (I, [I, I, DP, C.POINTER(C.c_float), V, V]),
        "addft_tc05_status": (C.c_uint, []),
        "addft_hpsi_fused_status": (C.c_uint, []),
        "addft_kinetic_stress": (I, [P, I, DP, I, DP, I, V, V, V, V, S, V]),
        "addft_density_gradients": (I, [P, P, DP, D, I, DP, C.POINTER(Psp), V, V, V, S, V]),
        "addft_nonlocal_gradients": (I, [P, I, DP, D, I, DP, I, I, DP, C.POINTER(Psp), V, V, V, V, V, S, V]),
        "addft_ffi_xc_lda": (I, [I, V, V, V, V, S, V]),
        "addft_ffi_xc_lda_work_bytes": (S, []),
        "addft_ffi_scatter": (I, [I, I, I, I, V, V, V, V]),
        "addft_ffi_gather": (I, [I, I, I, I, V, V, V, V]),
        "addft_ffi_check_index": (I, [I, I, V, V, V]),
        "addft_ffi_eigh_lowest": (I, [I, I, I, V, V, V, V, S, V]),
        "addft_ffi_eigh_lowest_work_bytes": (S, [I, I]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def _preload_torch_linalg() -> None:
    """Load torch's CUDA linear-algebra library by absolute path.

    torch opens ``libtorch_cuda_linalg.so`` lazily, by bare file name, on the
    first cuSOLVER call (eigh / cholesky in the solver).  A name-only dlopen
    depends on the calling object's search path, which process injectors
    (profilers) can change, so the first eigh then fails.  Once loaded here,
    the later dlopen by name finds the already-loaded object.
    """
    try:
        import torch
    except ImportError:
        return
    lib = Path(torch.__file__).resolve().parent / "lib" / "libtorch_cuda_linalg.so"
    if lib.exists():
        C.CDLL(str(lib), mode=C.RTLD_GLOBAL)


LIB = _load()
_preload_torch_linalg()

#: every C-ABI symbol declared in include/addft_gb300.h
EXPORTED = [
    "addft_status_string", "addft_last_error", "addft_version", "addft_launch_count", "addft_plan_create",
    "addft_plan_destroy", "addft_plan_info", "addft_work_bytes", "addft_psi_to_real",
    "addft_real_to_psi", "addft_kinetic", "addft_hpsi", "addft_becp", "addft_vnl_apply",
    "addft_nonlocal_energy", "addft_projectors", "addft_density", "addft_xc_lda",
    "addft_xc_lda_vjp", "addft_hartree", "addft_local_potential", "addft_ewald",
    "addft_kinetic_stress", "addft_density_gradients", "addft_nonlocal_gradients",
    "addft_hpsi_work_bytes", "addft_hartree_work_bytes", "addft_local_potential_work_bytes",
    "addft_density_gradients_work_bytes", "addft_nonlocal_gradients_work_bytes",
    "addft_ewald_work_bytes", "addft_occupations", "addft_hpsi_noalloc",
    "addft_hpsi_noalloc_max_scratch_bytes", "addft_kerker", "addft_kerker_work_bytes",
    "addft_plan_set_tuning", "addft_plan_get_tuning", "addft_zgemm_df", "addft_zgemm_df_work_bytes",
    "addft_peak_flops", "addft_tc05_status", "addft_ffi_xc_lda", "addft_ffi_xc_lda_work_bytes",
    "addft_ffi_scatter", "addft_ffi_gather", "addft_ffi_check_index", "addft_ffi_eigh_lowest",
    "addft_ffi_eigh_lowest_work_bytes", "addft_hpsi_fused_status", "addft_hpsi_host",
    "addft_hpsi_host_work_bytes",
]


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = LIB.addft_last_error().decode(errors="replace")
        name = LIB.addft_status_string(status).decode()
        raise AddftError(f"{what or 'addft'}: {name} ({status}): {msg}")


def dbl_array(values):
    vals = [float(v) for v in values]
    return (C.c_double * max(len(vals), 1))(*vals)
