"""ctypes binding of libeigenfns_gb300.so (the C ABI in include/eigenfns_gb300.h).

The library is the only compute path: importing a module that needs it raises
if the shared object is missing or fails to load. Nothing here falls back to a
CPU implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libeigenfns_gb300.so"

EF_OK = 0
EF_ERR_INVALID = 1
EF_ERR_UNSUPPORTED = 2
EF_ERR_CUDA = 3
EF_ERR_WORKSPACE = 4
EF_ERR_NONFINITE = 5
EF_ERR_TOO_LARGE = 6

EF_RAND_NORMAL = 0
EF_RAND_RADEMACHER = 1
EF_RAND_RADEMACHER_C = 2

_vp, _i, _ll, _d, _f, _sz, _u64 = C.c_void_p, C.c_int, C.c_longlong, C.c_double, C.c_float, C.c_size_t, C.c_uint64

# name -> (restype, argtypes); mirrors include/eigenfns_gb300.h
SIGNATURES = {
    "ef_version": (C.c_char_p, []),
    "ef_status_string": (C.c_char_p, [_i]),
    "ef_last_error": (C.c_char_p, []),
    "ef_launch_count": (C.c_ulonglong, []),
    "ef_supported_grid": (_i, [_i]),
    "ef_op_create": (_i, [_i, _d, _d, _d, _d, _vp, C.POINTER(_vp)]),
    "ef_op_destroy": (_i, [_vp]),
    "ef_op_configure": (_i, [_vp, _i, _sz]),
    "ef_op_pipeline": (_i, [_vp]),
    "ef_op_info": (_i, [_vp, C.POINTER(_i), C.POINTER(_d), C.POINTER(_d)]),
    "ef_op_basis": (_i, [_vp, _vp, _vp, _vp]),
    "ef_op_mask": (_i, [_vp, _vp, _vp]),
    "ef_op_workspace_bytes": (_sz, [_vp, _i]),
    "ef_theta": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ef_precondition": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ef_precondition_simple": (_i, [_vp, _vp, _vp, _i, _f, _vp]),
    "ef_h_realspace": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ef_e_realspace": (_i, [_vp, _vp, _vp, _vp, _i, _vp]),
    "ef_cheb_first": (_i, [_vp, _vp, _vp, _vp, _i, _d, _f, _f, _vp, _sz, _vp]),
    "ef_cheb_step": (_i, [_vp, _vp, _vp, _vp, _i, _d, _f, _vp, _sz, _vp]),
    "ef_kpm_first": (_i, [_vp, _vp, _vp, _i, _d, _vp, _i, _vp, _sz, _vp]),
    "ef_kpm_step": (_i, [_vp, _vp, _vp, _i, _d, _i, _vp, _i, _vp, _sz, _vp]),
    "ef_kpm_count_first": (_i, [_vp, _vp, _vp, _i, _d, _d, _d, _vp, _vp, _sz, _vp]),
    "ef_kpm_count_step": (_i, [_vp, _vp, _vp, _vp, _i, _d, _d, _vp, _vp, _sz, _vp]),
    "ef_gram_workspace_bytes": (_sz, [_i, _i, _ll]),
    "ef_gram": (_i, [_vp, _vp, _i, _i, _ll, _vp, _vp, _sz, _vp]),
    "ef_gram_noalloc": (_i, [_vp, _vp, _i, _i, _ll, _vp, _vp]),
    "ef_gram_tc_workspace_bytes": (_sz, [_i, _i, _ll]),
    "ef_tc_error": (_i, [_vp]),
    "ef_tc_error_async": (_i, [_vp, _vp]),
    "ef_group_theta": (_i, [_vp, _vp, _i, _vp, _ll, _vp, _ll, _i, _vp, _sz, _vp]),
    "ef_group_precondition": (_i, [_vp, _vp, _i, _vp, _ll, _vp, _ll, _i, _vp, _sz, _vp]),
    "ef_group_gram": (_i, [_vp, _i, _vp, _ll, _vp, _ll, _i, _i, _ll, _vp, _ll, _vp, _sz, _vp]),
    "ef_group_rotate": (_i, [_vp, _i, _vp, _ll, _vp, _ll, _vp, _ll, _i, _i, _ll, _i, _vp]),
    "ef_group_rowstats": (_i, [_vp, _i, _vp, _ll, _vp, _ll, _i, _ll, _vp, _ll, _vp, _sz, _vp]),
    "ef_group_residual_norms": (_i, [_vp, _i, _vp, _ll, _vp, _ll, _vp, _ll, _vp, _ll, _i, _ll,
                                     _vp, _ll, _vp, _sz, _vp]),
    "ef_group_scale_rows": (_i, [_vp, _i, _vp, _ll, _vp, _ll, _i, _ll, _vp]),
    "ef_tune_gram": (_i, [_i, _i, _i, _i]),
    "ef_tune_reset": (_i, []),
    "ef_energy_workspace_bytes": (_i, [_vp, _i]),
    "ef_energy_density": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ef_gram_tc": (_i, [_vp, _vp, _i, _i, _ll, _vp, _vp, _vp, _sz, _vp]),
    "ef_rotate": (_i, [_vp, _vp, _vp, _i, _i, _ll, _i, _vp]),
    "ef_fma_probe_flops": (C.c_longlong, [_i, _i]),
    "ef_fma_probe": (_i, [_vp, _i, _i, _i, _vp]),
    "ef_cholqr_f64": (_i, [_vp, _i, _i, _vp, _vp, _d, _vp]),
    "ef_eigh_f64_workspace_bytes": (_sz, [_i, _i]),
    "ef_eigh_f64": (_i, [_vp, _i, _i, _vp, _vp, _vp, _sz, _vp, _vp]),
    "ef_rowdot_workspace_bytes": (_sz, [_i, _ll]),
    "ef_rowdot": (_i, [_vp, _vp, _i, _ll, _vp, _vp, _sz, _vp]),
    "ef_rowstats": (_i, [_vp, _vp, _i, _ll, _vp, _vp, _sz, _vp]),
    "ef_residual": (_i, [_vp, _vp, _vp, _vp, _i, _ll, _vp]),
    "ef_residual_norms": (_i, [_vp, _vp, _vp, _vp, _i, _ll, _vp, _vp, _sz, _vp]),
    "ef_scale_rows": (_i, [_vp, _vp, _i, _ll, _vp]),
    "ef_axpby": (_i, [_vp, _vp, _ll, _d, _d, _vp]),
    "ef_rand_block": (_i, [_vp, _vp, _i, _u64, _u64, _i, _vp]),
    "ef_apply_mask": (_i, [_vp, _vp, _i, _vp]),
    "ef_rasterize_rods": (_i, [_i, _d, _vp, _i, _i, _d, _d, _vp]),
}

_lib = None


def load() -> C.CDLL:
    """Load the library once (torch's CUDA runtime is loaded first so both share it)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"eigenfns_gb300 CUDA library not found at {LIB_PATH}; build it with "
            "`python -m eigenfns_gb300.build` (or __graft_entry__.build())")
    import torch  # noqa: F401  (loads libcudart before the library resolves it)
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class EigenfnsError(RuntimeError):
    pass


def check(status: int, what: str = "") -> None:
    if status == EF_OK:
        return
    lib = load()
    msg = f"{what}: {lib.ef_status_string(status).decode()} ({lib.ef_last_error().decode()})"
    if status in (EF_ERR_INVALID, EF_ERR_UNSUPPORTED, EF_ERR_WORKSPACE, EF_ERR_NONFINITE,
                  EF_ERR_TOO_LARGE):
        raise ValueError(msg)
    raise EigenfnsError(msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
