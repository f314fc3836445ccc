"""ctypes binding of libnbkdt.so (the C ABI declared in include/nbkdt.h).

The library must exist in-tree (built by ``nbodylib_gb300._build.build()`` or
``__graft_entry__.build()``); there is no fallback: loading fails loudly without it.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

_LIB = None

c_int = ctypes.c_int
c_i32p = ctypes.POINTER(ctypes.c_int32)
c_i64 = ctypes.c_int64
c_i64p = ctypes.POINTER(ctypes.c_int64)
c_dbl = ctypes.c_double
c_dblp = ctypes.POINTER(ctypes.c_double)
c_vp = ctypes.c_void_p

# name: (restype, argtypes)
SIGNATURES = {
    "nbk_last_error": (ctypes.c_char_p, []),
    "nbk_version": (ctypes.c_char_p, []),
    "nbk_launch_count": (ctypes.c_longlong, []),
    "nbk_probe_fp64": (c_int, [c_dblp]),
    "nbk_trace_enable": (c_int, [c_int]),
    "nbk_trace_reset": (c_int, []),
    "nbk_trace_json": (c_i64, [ctypes.c_char_p, c_i64]),
    "nbk_kernel_binary_version": (c_int, [ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "nbk_debug_set_iteration_cap": (c_int, [c_int]),
    "nbk_debug_fail_allocation": (c_int, [ctypes.c_longlong]),
    "nbk_debug_live_allocations": (ctypes.c_longlong, []),
    "nbk_create": (c_int, [c_vp, c_vp, c_vp, c_i64, c_int, c_int, c_int, c_int, c_int, c_int,
                           c_int, c_vp, ctypes.c_uint, ctypes.POINTER(c_vp)]),
    "nbk_destroy": (c_int, [c_vp]),
    "nbk_set_stream": (c_int, [c_vp, c_vp]),
    "nbk_sync": (c_int, [c_vp]),
    "nbk_get_counts": (c_int, [c_vp, c_i64p, c_i64p, c_i64p, c_i32p]),
    "nbk_get_perm": (c_int, [c_vp, c_vp]),
    "nbk_get_kernel": (c_int, [c_vp, c_vp, c_dblp]),
    "nbk_knn": (c_int, [c_vp, c_int, c_int, c_int, c_vp, c_vp]),
    "nbk_knn_points": (c_int, [c_vp, c_vp, c_i64, c_int, c_int, c_vp, c_vp]),
    "nbk_knn_coords": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp]),
    "nbk_knn_phase_points": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp]),
    "nbk_knn_targets": (c_int, [c_vp, c_vp, c_i64, c_int, c_int, c_int, c_vp, c_vp]),
    "nbk_density": (c_int, [c_vp, c_int, c_vp]),
    "nbk_density_noalloc": (c_int, [c_vp, c_int, c_vp]),
    "nbk_density_particles": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp]),
    "nbk_veldensity": (c_int, [c_vp, c_int, c_int, c_vp]),
    "nbk_density_veldensity": (c_int, [c_vp, c_int, c_int, c_vp, c_vp]),
    "nbk_veldensity_particles": (c_int, [c_vp, c_vp, c_i64, c_int, c_int, c_vp]),
    "nbk_density_points": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp]),
    "nbk_veldensity_points": (c_int, [c_vp, c_vp, c_vp, c_i64, c_int, c_int, c_vp]),
    "nbk_smooth_vel": (c_int, [c_vp, c_int, c_vp, c_vp]),
    "nbk_smooth_vel_disp": (c_int, [c_vp, c_int, c_vp, c_vp, c_vp]),
    "nbk_smooth_vel_skew": (c_int, [c_vp, c_int, c_vp, c_vp, c_vp, c_vp]),
    "nbk_smooth_vel_kurtosis": (c_int, [c_vp, c_int, c_vp, c_vp, c_vp, c_vp]),
    "nbk_veldensity_physdensity": (c_int, [c_vp, c_int, c_int, c_vp, c_vp]),
    "nbk_veldensity_physdensity_particles": (c_int, [c_vp, c_vp, c_i64, c_int, c_int, c_vp, c_vp]),
    "nbk_smooth_vel_particles": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp]),
    "nbk_smooth_vel_points": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp]),
    "nbk_smooth_vel_disp_particles": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp, c_vp]),
    "nbk_smooth_vel_disp_points": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp, c_vp]),
    "nbk_smooth_local_mean_particles": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp, c_vp]),
    "nbk_smooth_local_mean_points": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp, c_vp]),
    "nbk_smooth_local_disp_particles": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp, c_vp,
                                                c_vp]),
    "nbk_smooth_local_disp_points": (c_int, [c_vp, c_vp, c_i64, c_int, c_vp, c_vp, c_vp, c_vp]),
    "nbk_ball_tagged": (c_int, [c_vp, c_vp, c_i64, c_dbl, c_vp, c_vp, c_i64, c_i64p]),
    "nbk_ball_tagged_points": (c_int, [c_vp, c_vp, c_i64, c_dbl, c_vp, c_vp, c_i64, c_i64p]),
    "nbk_ball_mark": (c_int, [c_vp, ctypes.c_int32, c_dbl, ctypes.c_int32, c_vp, c_vp]),
    "nbk_fof": (c_int, [c_vp, c_dbl, ctypes.c_int32, c_int, c_vp, c_i32p]),
    "nbk_fof_criterion": (c_int, [c_vp, c_int, c_vp, ctypes.c_int32, c_int, c_vp, c_i32p]),
    "nbk_fof_nn_criterion": (c_int, [c_vp, c_int, c_vp, c_int, c_vp, ctypes.c_int32, c_vp,
                                     c_i32p]),
    "nbk_fof_nn_dist_criterion": (c_int, [c_vp, c_int, c_vp, c_int, c_vp, c_vp, c_int, c_vp,
                                          ctypes.c_int32, c_vp, c_i32p]),
    "nbk_density_adjoint": (c_int, [c_vp, c_int, c_vp, c_vp, c_vp, c_vp]),
    "nbk_batch_create": (c_int, [c_vp, c_vp, c_vp, c_i64, c_int, c_int, c_int, ctypes.c_uint,
                                 ctypes.POINTER(c_vp)]),
    "nbk_batch_destroy": (c_int, [c_vp]),
    "nbk_batch_set_stream": (c_int, [c_vp, c_vp]),
    "nbk_batch_density": (c_int, [c_vp, c_int, c_vp, c_int]),
    "nbk_batch_density_pertree": (c_int, [c_vp, c_int, c_vp]),
    "nbk_batch_density_pertree_search": (c_int, [c_vp, c_int, c_vp]),
    "nbk_batch_set_query_mapping": (c_int, [c_vp, c_int]),
    "nbk_batch_get_query_mapping": (c_int, [c_vp, c_i32p]),
    "nbk_batch_get_params": (c_int, [c_vp, c_i32p, c_i32p, ctypes.c_char_p, c_i64]),
}

STATUS = {0: "NBK_OK", 1: "NBK_ERR_INVALID", 2: "NBK_ERR_UNSUPPORTED", 3: "NBK_ERR_CUDA",
          4: "NBK_ERR_NOMEM", 5: "NBK_ERR_TOO_FEW", 6: "NBK_ERR_DEVICE"}


class NbkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def lib_path() -> str:
    return _build.LIB


def load() -> ctypes.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError(
            f"libnbkdt.so is not built ({path}); run nbodylib_gb300._build.build() first. "
            "There is no CPU fallback for the KDTree kernels.")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != 0:
        msg = load().nbk_last_error().decode(errors="replace")
        raise NbkError(status, msg)
