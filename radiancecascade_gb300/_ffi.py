"""ctypes bindings of include/rc.h (librc.so, built in-tree by build.py).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "librc.so")

RC_OK, RC_ERR_INVALID_ARG, RC_ERR_OOM, RC_ERR_CUDA, RC_ERR_TIMEOUT, RC_ERR_UNSUPPORTED, RC_ERR_STATE = range(7)
RC_PRECISION_FP32, RC_PRECISION_FP16 = 0, 1
RC_MEM_HOST, RC_MEM_DEVICE = 0, 1

VOXEL_DT = np.dtype([("emission", "<u2", (3,)), ("albedo_occ", "<u2")])
BOX_DT = np.dtype([("lo", "<i4", (3,)), ("hi", "<i4", (3,)), ("value", VOXEL_DT)])
SPHERE_DT = np.dtype([("centre", "<f8", (3,)), ("radius", "<f8"), ("velocity", "<f8", (3,)),
                      ("value", VOXEL_DT), ("pad", "<u4", (2,))])
OPAQUE = 0x8000


class Params(C.Structure):
    _fields_ = [("grid", C.c_int32 * 3), ("num_cascades", C.c_int32), ("probe_spacing0", C.c_int32),
                ("dir_res0", C.c_int32), ("interval0", C.c_int32), ("interval_ratio", C.c_int32),
                ("precision", C.c_int32), ("reserved", C.c_int32 * 7)]


class SceneSpec(C.Structure):
    _fields_ = [("grid", C.c_int32 * 3), ("num_boxes", C.c_int32), ("box_edge_min", C.c_int32),
                ("box_edge_max", C.c_int32), ("num_spheres", C.c_int32), ("reserved", C.c_int32),
                ("albedo_min", C.c_double), ("albedo_max", C.c_double), ("radius_min", C.c_double),
                ("radius_max", C.c_double), ("emission_min", C.c_double), ("emission_max", C.c_double),
                ("speed", C.c_double)]


class LevelInfo(C.Structure):
    _fields_ = [("probes", C.c_int32 * 3), ("spacing", C.c_int32), ("dir_res", C.c_int32),
                ("num_dirs", C.c_int32), ("interval_lo", C.c_int32), ("interval_hi", C.c_int32),
                ("radiance_elems", C.c_int64), ("radiance_bytes", C.c_int64)]


class NrcParams(C.Structure):
    _fields_ = [("first_level", C.c_int32), ("hash_log2_entries", C.c_int32), ("base_resolution", C.c_int32),
                ("max_resolution", C.c_int32), ("learning_rate", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("epsilon", C.c_float), ("train_fraction_log2", C.c_int32),
                ("steps_per_solve", C.c_int32), ("fallback_threshold", C.c_float), ("fallback_tile", C.c_int32),
                ("radiance_scale", C.c_float), ("plain_level_fraction", C.c_float), ("seed", C.c_uint64)]


class NrcStats(C.Structure):
    _fields_ = [("solves", C.c_int64), ("steps", C.c_int64), ("last_loss", C.c_float), ("served_levels", C.c_int32),
                ("fallback_tiles", C.c_int64), ("tiles", C.c_int64), ("served_solves", C.c_int64 * 10)]


class ShadeMaterial(C.Structure):
    _fields_ = [("ambient", C.c_float * 4), ("diffuse", C.c_float * 4), ("specular", C.c_float * 4),
                ("shininess", C.c_float), ("enable_bit", C.c_uint32), ("color_texture", C.c_int32),
                ("normal_texture", C.c_int32)]


class Texture(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("srgb", C.c_int32),
                ("pad", C.c_int32)]


class ShadeView(C.Structure):
    _fields_ = [("view_proj", C.c_float * 16), ("eye", C.c_float * 3), ("light", C.c_float * 3),
                ("width", C.c_int32), ("height", C.c_int32), ("world_to_grid", C.c_float * 12),
                ("gi_scale", C.c_float), ("pad", C.c_int32)]


class BatchTiles(C.Structure):
    _fields_ = [("probes_per_item", C.c_int32), ("dirs_per_item", C.c_int32), ("blocks_per_item", C.c_int32),
                ("walks_per_item", C.c_int32)]


_P = C.c_void_p
_S = C.c_int  # rc_status

# name -> (restype, argtypes); the full ABI of include/rc.h
SIGNATURES = {
    "rc_status_string": (C.c_char_p, [C.c_int]),
    "rc_last_error": (C.c_char_p, []),
    "rc_abi_version": (C.c_int, []),
    "rc_params_default": (_S, [_P, C.c_int32, C.c_int32]),
    "rc_params_validate": (_S, [_P]),
    "rc_level_info_get": (_S, [_P, C.c_int32, _P]),
    "rc_fluence_elems": (C.c_int64, [_P]),
    "rc_scene_generate": (_S, [_P, C.c_uint64, _P, _P]),
    "rc_spheres_advance": (_S, [_P, C.c_int32, _P, C.c_int32]),
    "rc_voxelise_host": (_S, [_P, _P, C.c_int32, _P, C.c_int32, _P]),
    "rc_directions": (_S, [C.c_int32, _P]),
    "rc_solid_angles": (_S, [C.c_int32, _P]),
    "rc_create": (_S, [_P, C.c_int32, C.POINTER(C.c_void_p)]),
    "rc_destroy": (_S, [_P]),
    "rc_get_params": (_S, [_P, _P]),
    "rc_scene_upload": (_S, [_P, _P, C.c_int64, C.c_int32]),
    "rc_scene_set_boxes": (_S, [_P, _P, C.c_int32]),
    "rc_scene_set_spheres": (_S, [_P, _P, C.c_int32]),
    "rc_solve": (_S, [_P, _P]),
    "rc_synchronize": (_S, [_P]),
    "rc_get_fluence": (_S, [_P, _P, C.c_int64, C.c_int32]),
    "rc_get_radiance": (_S, [_P, C.c_int32, _P, C.c_int64, C.c_int32]),
    "rc_fluence_device_ptr": (_S, [_P, C.POINTER(C.c_void_p)]),
    "rc_radiance_device_ptr": (_S, [_P, C.c_int32, C.POINTER(C.c_void_p)]),
    "rc_get_stream": (_S, [_P, C.POINTER(C.c_void_p)]),
    "rc_profile_levels": (_S, [_P, C.c_int32, _P, C.c_int32]),
    "rc_solve_noalloc": (_S, [_P, _P, _P, _P, _P]),
    "rc_get_fluence_async": (_S, [_P, _P, C.c_int64]),
    "rc_scene_set_mesh": (_S, [_P, _P, C.c_int64, _P, C.c_int64, _P, _P, C.c_int32]),
    "rc_get_volume": (_S, [_P, _P, C.c_int64, C.c_int32]),
    "rc_shade": (_S, [_P, C.POINTER(ShadeView), _P, C.c_int64, _P, C.c_int64, _P, C.POINTER(ShadeMaterial),
                      C.c_int32, C.POINTER(Texture), C.c_int32, _P, C.c_int32]),
    "rc_shade_set_mesh": (_S, [_P, _P, C.c_int64, _P, C.c_int64, _P, C.POINTER(ShadeMaterial), C.c_int32,
                               C.POINTER(Texture), C.c_int32]),
    "rc_shade_draw": (_S, [_P, C.POINTER(ShadeView), _P, C.c_int32]),
    "rc_batch_create": (_S, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "rc_batch_destroy": (_S, [_P]),
    "rc_batch_scene_set": (_S, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int32]),
    "rc_batch_solve": (_S, [_P, _P]),
    "rc_batch_synchronize": (_S, [_P]),
    "rc_batch_get_fluence": (_S, [_P, C.c_int32, _P, C.c_int64, C.c_int32]),
    "rc_batch_get_radiance": (_S, [_P, C.c_int32, C.c_int32, _P, C.c_int64, C.c_int32]),
    "rc_batch_set_spheres": (_S, [_P, C.c_int32, _P, C.c_int32]),
    "rc_set_stage_timing": (_S, [_P, C.c_int32]),
    "rc_check_status": (_S, [C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]),
    "rc_get_stage_ms": (_S, [_P, _P, C.c_int32]),
    "rc_batch_get_fluence_all": (_S, [_P, _P, C.c_int64, C.c_int32]),
    "rc_batch_get_fluence_all_async": (_S, [_P, _P, C.c_int64]),
    "rc_batch_set_tiles": (_S, [_P, C.POINTER(BatchTiles)]),
    "rc_batch_get_tiles": (_S, [_P, C.POINTER(BatchTiles)]),
    "rc_batch_get_form": (_S, [_P, C.POINTER(C.c_int32)]),
    "rc_batch_tune": (_S, [_P, C.c_int32, C.POINTER(BatchTiles), C.POINTER(C.c_float)]),
    "rc_nrc_param_count": (C.c_int32, []),
    "rc_nrc_params_default": (_S, [C.POINTER(NrcParams)]),
    "rc_nrc_enable": (_S, [_P, C.POINTER(NrcParams)]),
    "rc_nrc_disable": (_S, [_P]),
    "rc_nrc_save": (_S, [_P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "rc_nrc_load": (_S, [_P, _P, C.c_int64]),
    "rc_nrc_get_stats": (_S, [_P, C.POINTER(NrcStats)]),
    "rc_nrc_query": (_S, [_P, C.c_int32, _P, _P, C.c_int64, _P]),
    "rc_nrc_tile_gradient": (_S, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P]),
}

_lib = None


class RCError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (status_name(status), message))
        self.status = status
        self.message = message


def lib() -> C.CDLL:
    """Load librc.so (or the library RC_LIBRARY names, e.g. the checked build
    librc_checked.so).  Raises (never falls back) when it was not built."""
    global _lib
    if _lib is None:
        path = os.environ.get("RC_LIBRARY") or LIB_PATH
        if not os.path.exists(path):
            raise ImportError("%s is missing: build it first "
                              "(python -m radiancecascade_gb300.build or __graft_entry__.build())" % path)
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_name(s: int) -> str:
    try:
        return lib().rc_status_string(s).decode()
    except Exception:  # pragma: no cover - library not loadable
        return "RC_STATUS_%d" % s


def last_error() -> str:
    return lib().rc_last_error().decode(errors="replace")


def check(status: int) -> None:
    if status != RC_OK:
        raise RCError(status, last_error())


def ptr(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)
