"""ctypes binding of the C ABI declared in include/ccs_gpu.h.

The library is the in-tree ``_build/libccs_gpu.so``; importing this module fails
loudly when it has not been built (there is no CPU fallback for the step).  The
environment variable CCS_GPU_LIB selects another in-tree build of the same ABI (the
bounds-checked ``_build/bounds/libccs_gpu.so``) for a whole process.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(os.environ.get("CCS_GPU_LIB") or Path(__file__).resolve().parent / "_build" / "libccs_gpu.so")

CCS_OK = 0
CCS_ERR_ARG = 1
CCS_ERR_CUDA = 2
CCS_ERR_NAN = 3
CCS_ERR_TIMEOUT = 4
CCS_ERR_UNSUPPORTED = 5
CCS_ERR_MESH = 6
CCS_ERR_NOMEM = 7
CCS_ERR_NODEVICE = 8
CCS_ERR_TOO_LARGE = 9
CCS_ERR_IO = 10
CCS_NOALLOC_MAX_N = 4096

CCS_RK4 = 0
CCS_RK3_TVD = 1
CCS_FP64 = 0
CCS_MIXED = 1
CCS_EDISS_ZERO = 0
CCS_EDISS_RECONSTRUCT = 1
CCS_MAX_VARIANTS = 4
# mixed-lane variants: (tile_x, tile_y, halo-staging schedule)
MIXED_VARIANTS = ((32, 32, "loads"), (32, 16, "loads"), (32, 32, "async"), (32, 16, "async"))
CCS_OP_WENO, CCS_OP_CENTRAL2, CCS_OP_CENTRAL4, CCS_OP_CENTRAL6 = 0, 2, 4, 6
CCS_MAP_GNOMONIC_EQUIANGULAR = 0
CCS_MAP_CONFORMAL = 1
CCS_MESH_POLE_INVERSE = 1
CCS_IC_CASE2 = 2
CCS_IC_CASE5 = 5
CCS_IC_CASE6 = 6
CCS_IC_SEEDED = 100

_dp = C.POINTER(C.c_double)


class Config(C.Structure):
    _fields_ = [
        ("N", C.c_int), ("halo", C.c_int), ("scheme", C.c_int), ("precision", C.c_int),
        ("e_dissipation", C.c_int), ("device", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dt", C.c_double),
        ("radius", C.c_double), ("gravity", C.c_double), ("omega", C.c_double),
        ("phi_mean", C.c_double),
    ]


class MeshView(C.Structure):
    _fields_ = [(n, _dp) for n in ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "phis")]


STATE_FIELDS = ("phiG", "u", "v", "phi", "uC", "vC", "zonal_wind", "meridional_wind", "phit")


class StateView(C.Structure):
    _fields_ = [(n, _dp) for n in STATE_FIELDS]


class ICParams(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("lmax_h", C.c_int), ("lmax_psi", C.c_int), ("lmax_oro", C.c_int),
        ("seed", C.c_uint64),
        ("h0", C.c_double), ("h_rms", C.c_double), ("wind_max", C.c_double),
        ("oro_rms", C.c_double), ("oro_max", C.c_double),
    ]


# name -> (restype, argtypes); every symbol include/ccs_gpu.h declares
_vp = C.c_void_p
SIGNATURES = {
    "ccs_init": (C.c_int, [C.POINTER(Config), C.POINTER(MeshView), C.POINTER(_vp)]),
    "ccs_init_shared": (C.c_int, [C.POINTER(Config), _vp, C.POINTER(_vp)]),
    "ccs_destroy": (None, [_vp]),
    "ccs_set_state": (C.c_int, [_vp, C.POINTER(StateView)]),
    "ccs_get_state": (C.c_int, [_vp, C.POINTER(StateView)]),
    "ccs_set_state_async": (C.c_int, [_vp, C.POINTER(StateView)]),
    "ccs_get_state_async": (C.c_int, [_vp, C.POINTER(StateView)]),
    "ccs_step": (C.c_int, [_vp, C.c_int]),
    "ccs_step_async": (C.c_int, [_vp, C.c_int]),
    "ccs_sync": (C.c_int, [_vp]),
    "ccs_spatial_operator": (C.c_int, [_vp, _dp, _dp, _dp]),
    "ccs_set_operator": (C.c_int, [_vp, C.c_int]),
    "ccs_check_state": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "ccs_autotune": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_int), _dp]),
    "ccs_set_variant": (C.c_int, [_vp, C.c_int]),
    "ccs_get_variant": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ccs_diag": (C.c_int, [_vp, _dp, _dp]),
    "ccs_diag_noalloc": (C.c_int, [C.c_int, C.c_int] + [C.c_void_p] * 9 + [_vp]),
    "ccs_batch_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.POINTER(_vp)]),
    "ccs_batch_step": (C.c_int, [_vp, C.c_int]),
    "ccs_batch_step_async": (C.c_int, [_vp, C.c_int]),
    "ccs_batch_stream": (C.c_void_p, [_vp]),
    "ccs_batch_destroy": (None, [_vp]),
    "ccs_batch_autotune": (C.c_int, [_vp, C.c_int]),
    "ccs_batch_info": (C.c_int, [_vp, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int)]),
    "ccs_batch_last_error": (C.c_char_p, [_vp]),
    "ccs_ghost_map": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int64)]),
    "ccs_timing": (C.c_int, [_vp, C.c_int, C.c_int, _dp, C.POINTER(C.c_int64)]),
    "ccs_stream": (C.c_void_p, [_vp]),
    "ccs_selftest_div": (C.c_int, [_dp, C.c_int64, C.c_double, _dp, _dp]),
    "ccs_selftest_div_pairs": (C.c_int, [_dp, _dp, C.c_int64, _dp, _dp]),
    "ccs_debug_bounds": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
    "ccs_courant": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ccs_debug_bounds_selftest": (C.c_int, []),
    "ccs_strerror": (C.c_char_p, [C.c_int]),
    "ccs_mesh_save": (C.c_int, [C.c_char_p, C.c_int, C.c_int] + [_dp] * 6),
    "ccs_mesh_file_info": (C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ccs_mesh_load": (C.c_int, [C.c_char_p, C.c_int] + [_dp] * 6),
    "ccs_state_write": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(StateView)]),
    "ccs_state_read": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(StateView)]),
    "ccs_last_error": (C.c_char_p, [_vp]),
    "ccs_abi_version": (C.c_int, []),
    "ccs_mesh_generate": (C.c_int, [C.c_int, C.c_int] + [_dp] * 6),
    "ccs_mesh_derive": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 16),
    "ccs_mesh_derive_ex": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int] + [_dp] * 16),
    "ccs_initial_condition": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                        C.POINTER(ICParams)] + [_dp] * 8),
    "ccs_state_from_sphere": (C.c_int, [C.c_int, C.c_int, C.POINTER(MeshView), C.POINTER(StateView)]),
    "ccs_cfl_dt": (C.c_double, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                C.POINTER(MeshView), C.POINTER(StateView)]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded library (raises if it is missing: build it with build.build())."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: the CUDA library must be built (conformal_cubed_sphere_gb300.build)")
        _lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


class CCSError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {lib().ccs_strerror(status).decode()} ({status})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


def check(status: int, where: str, handle=None) -> None:
    if status != CCS_OK:
        detail = ""
        if handle is not None:
            detail = (lib().ccs_last_error(handle) or b"").decode()
        raise CCSError(status, where, detail)
