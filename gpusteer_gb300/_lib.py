"""ctypes binding of libgpusteer.so (include/gpusteer.h).

The library is built in-tree (gpusteer_gb300/_build/).  Loading fails loudly
when it is missing and cannot be built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

_lock = threading.Lock()
_lib = None

_u = C.c_uint
_f = C.c_float
_i = C.c_int
_vp = C.c_void_p
_fp = C.POINTER(C.c_float)
_up = C.POINTER(C.c_uint)

GS_OK = 0
STATUS_NAMES = {0: "GS_OK", 1: "GS_ERR_INVALID_ARG", 2: "GS_ERR_OOM", 3: "GS_ERR_CUDA",
                4: "GS_ERR_TIMEOUT", 5: "GS_ERR_NONFINITE", 6: "GS_ERR_STATE",
                7: "GS_ERR_UNSUPPORTED"}


class GpuSteerError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class AgentArrays(C.Structure):
    _fields_ = [("position", _fp), ("direction", _fp), ("steering", _fp), ("side", _fp),
                ("up", _fp), ("speed", _fp), ("max_speed", _fp), ("max_force", _fp),
                ("radius", _fp), ("mass", _fp), ("applied", _up)]


class StepParams(C.Structure):
    _fields_ = [
        ("world_size", _f * 3), ("world_cells", _u * 3), ("search_radius", _u),
        ("wrap_mode", _i), ("knn_mode", _i), ("k", _u), ("clear_applied", _i),
        ("knw", _u), ("min_time_to_wall", _f), ("w_walls", _f), ("mask_walls", _u),
        ("min_time_to_collision", _f), ("min_separation_distance", _f), ("avoid_close", _i),
        ("w_avoid", _f), ("mask_avoid", _u),
        ("sep_min", _f), ("sep_max", _f), ("sep_cos", _f), ("w_sep", _f), ("mask_sep", _u),
        ("ali_min", _f), ("ali_max", _f), ("ali_cos", _f), ("w_ali", _f), ("mask_ali", _u),
        ("coh_min", _f), ("coh_max", _f), ("coh_cos", _f), ("w_coh", _f), ("mask_coh", _u),
        ("seek_target", _f * 3), ("w_seek", _f), ("mask_seek", _u),
        ("order", _u * 8), ("n_order", _u), ("dt", _f),
        ("path", _vp), ("path_prediction_time", _f), ("w_path", _f), ("mask_path", _u),
    ]


# name -> argtypes (all return gs_status unless listed in _RESTYPE)
SIGNATURES = {
    "gs_status_string": [_i],
    "gs_last_error": [],
    "gs_version": [],
    "gs_max_k": [],
    "gs_set_device": [_i],
    "gs_host_alloc": [C.c_size_t, C.POINTER(_vp)],
    "gs_host_free": [_vp],
    "gs_bins_create": [_up, _fp, _u, C.POINTER(_vp)],
    "gs_bins_destroy": [_vp],
    "gs_bins_num_cells": [_vp, _up],
    "gs_bins_get_cells": [_vp, _fp, _fp, _fp, _u],
    "gs_group_create": [_u, _u, _vp, C.POINTER(_vp)],
    "gs_group_destroy": [_vp],
    "gs_group_upload": [_vp, C.POINTER(AgentArrays), _u],
    "gs_group_download": [_vp, C.POINTER(AgentArrays)],
    "gs_group_size": [_vp, _up],
    "gs_group_device_arrays": [_vp, C.POINTER(AgentArrays)],
    "gs_group_stream": [_vp, C.POINTER(_vp)],
    "gs_group_synchronize": [_vp],
    "gs_group_set_profiling": [_vp, _i],
    "gs_group_phase_times": [_vp, _fp, _up, _u],
    "gs_group_exact_redos": [_vp, _up],
    "gs_group_set_persistent": [_vp, C.c_int],
    "gs_group_set_barrier_limit": [_vp, _u],
    "gs_knn_create": [_u, _u, C.POINTER(_vp)],
    "gs_knn_destroy": [_vp],
    "gs_knn_download": [_vp, _vp, _up, _fp],
    "gs_knn_device_arrays": [_vp, C.POINTER(_up), C.POINTER(_fp)],
    "gs_knn_upload": [_vp, _vp, _up, _fp],
    "gs_find_knn_groups": [C.POINTER(_vp), _u, _vp, C.POINTER(_vp)],
    "gs_multigroup_step": [C.POINTER(_vp), _u, _vp, C.POINTER(_vp), C.POINTER(_vp), _vp, _u],
    "gs_walls_create": [_fp, _fp, _fp, _u, _vp, _u, C.POINTER(_vp)],
    "gs_walls_load": [C.c_char_p, _vp, _u, C.POINTER(_vp)],
    "gs_walls_destroy": [_vp],
    "gs_walls_size": [_vp, _up],
    "gs_walls_download": [_vp, _fp, _fp, _fp, _fp, _u],
    "gs_wrap_world": [_vp, _fp, _i],
    "gs_update_knn_database": [_vp, _vp],
    "gs_walls_update_knn_database": [_vp, _vp],
    "gs_find_knn": [_vp, _vp, _vp, _vp, _u],
    "gs_find_knn_walls": [_vp, _vp, _vp, _vp, _u],
    "gs_knn_bruteforce": [_vp, _vp, _vp],
    "gs_knn_bruteforce_pairs": [_vp, C.POINTER(C.c_ulonglong)],
    "gs_steer_for_separation": [_vp, _vp, _vp, _f, _f, _f, _f, _u],
    "gs_steer_for_alignment": [_vp, _vp, _vp, _f, _f, _f, _f, _u],
    "gs_steer_for_cohesion": [_vp, _vp, _vp, _f, _f, _f, _f, _u],
    "gs_steer_for_seek": [_vp, _fp, _f, _u],
    "gs_steer_to_avoid_neighbors": [_vp, _vp, _vp, _f, _f, _i, _f, _u],
    "gs_steer_to_avoid_walls": [_vp, _vp, _vp, _f, _f, _u],
    "gs_update_group": [_vp, _f],
    "gs_anti_penetration_agents": [_vp, _vp, _vp, _u],
    "gs_update_group_with_antipenetration": [_vp, _vp, _vp, _f],
    "gs_anti_penetration_wall": [_vp, _vp, _vp, _f, _u],
    "gs_step": [_vp, _vp, _vp, C.POINTER(StepParams), _u],
    "gs_step_host": [_vp, _vp, _vp, C.POINTER(StepParams), _u, C.POINTER(AgentArrays), _u,
                     C.POINTER(AgentArrays)],
    "gs_group_set_graphs": [_vp, _i],
    "gs_group_set_block": [_vp, _u],
    "gs_group_set_knn_capacity": [_vp, _u],
    "gs_group_knn_capacity": [_vp, _up],
    "gs_batch_create": [_u, _up, _u, _up, _fp, _u, _vp, C.POINTER(_vp)],
    "gs_batch_destroy": [_vp],
    "gs_batch_set_walls": [_vp, _u, _fp, _fp, _fp, _u],
    "gs_batch_upload": [_vp, C.POINTER(AgentArrays)],
    "gs_batch_download": [_vp, C.POINTER(AgentArrays)],
    "gs_batch_group": [_vp, C.POINTER(_vp)],
    "gs_batch_step": [_vp, C.POINTER(StepParams), _u],
    "gs_knn_binned_noalloc": [_vp, _u, _up, _fp, _u, _u, _vp, _vp, _vp],
    "gs_cell_density": [_vp, _vp, _up],
    "gs_cell_avg_velocity": [_vp, _vp, _fp],
    "gs_batch_cell_density": [_vp, _up],
    "gs_batches_step_host": [C.POINTER(_vp), _u, _vp, _u, _vp, _vp],
    "gs_batch_cell_avg_velocity": [_vp, _fp],
    "gs_path_create": [_fp, _u, _f, _i, C.POINTER(_vp)],
    "gs_path_destroy": [_vp],
    "gs_path_get": [_vp, _fp, _fp, _fp, _u, _up, _fp],
    "gs_steer_to_follow_path": [_vp, _vp, _f, _f, _u],
    "gs_rollout_create": [_vp, _vp, _u, _u, C.POINTER(_vp)],
    "gs_rollout_destroy": [_vp],
    "gs_rollout_forward": [_vp, C.POINTER(StepParams)],
    "gs_rollout_backward": [_vp, _vp, _vp, _vp, _vp, _fp],
    "gs_flock_adjoint_step": [_vp, _vp, _vp, _u, _u, _vp, _vp, _vp, C.POINTER(StepParams), _vp,
                              _vp, _vp, _vp, _vp, _u, _vp],
}
_RESTYPE = {"gs_status_string": C.c_char_p, "gs_last_error": C.c_char_p, "gs_version": _i,
            "gs_max_k": _u}


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """The loaded library; builds it first when it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            path = library_path()
            if not path.exists():
                if not build_if_missing:
                    raise RuntimeError(f"{path} is missing; run gpusteer_gb300.build.build()")
                _build.build()
            lib = C.CDLL(str(path))
            for name, args in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = _RESTYPE.get(name, _i)
            _lib = lib
        return _lib


def check(status: int) -> None:
    if status != GS_OK:
        msg = load().gs_last_error()
        raise GpuSteerError(status, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
