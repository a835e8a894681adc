"""ctypes bindings of the C ABI in include/uslam.h.

Importing this module loads the in-tree ``libuslam.so``.  There is no CPU
fallback: if the library is missing, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libuslam.so")

OK, INVALID_ARG, OOM, TIMEOUT, CUDA_ERROR, CAPACITY, NOT_READY, KERNEL_CHECK = range(8)
STATUS_NAMES = {
    OK: "OK", INVALID_ARG: "INVALID_ARG", OOM: "OOM", TIMEOUT: "TIMEOUT", CUDA_ERROR: "CUDA_ERROR",
    CAPACITY: "CAPACITY", NOT_READY: "NOT_READY", KERNEL_CHECK: "KERNEL_CHECK",
}

# gpumodels::Feature (wslam/src/models.hpp:31-69), 48 bytes
FEATURE_DTYPE = np.dtype([
    ("x", "<f4"), ("y", "<f4"), ("strength", "<u4"), ("orientation", "<f4"), ("descriptor", "<u4", (8,)),
])
MATCH_DTYPE = np.dtype([("lod_a", "<i4"), ("idx_a", "<i4"), ("lod_b", "<i4"), ("idx_b", "<i4")])
assert FEATURE_DTYPE.itemsize == 48 and MATCH_DTYPE.itemsize == 16


class ServerParams(C.Structure):
    _fields_ = [
        ("n_sizes", C.c_int), ("widths", C.POINTER(C.c_int)), ("heights", C.POINTER(C.c_int)),
        ("hbm_budget_bytes", C.c_size_t), ("max_batch", C.c_int),
    ]


class Params(C.Structure):
    _fields_ = [
        ("device", C.c_int), ("levels", C.c_int), ("max_width", C.c_int), ("max_height", C.c_int),
        ("cap_per_level", C.c_int), ("brief_pattern", C.POINTER(C.c_int32)), ("matcher", C.c_int),
        ("ratio", C.c_float), ("cell_cap", C.c_int), ("detector", C.c_int), ("frame_cap", C.c_int),
        ("describe_form", C.c_int),
    ]


class Camera(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("fu", "fv", "cu", "cv", "k1", "k2", "p1", "p2")]


class TriOpts(C.Structure):
    _fields_ = [
        ("max_reprojection_px", C.c_double), ("min_depth", C.c_double), ("max_depth", C.c_double),
        ("undistort_tolerance", C.c_double), ("min_inliers", C.c_int), ("undistort_iterations", C.c_int),
    ]


# uslam_tri_result (128 bytes)
TRI_RESULT_DTYPE = np.dtype([
    ("rotation", "<f8", (9,)), ("translation", "<f8", (3,)), ("mean_reprojection_error_px", "<f8"),
    ("rotation_angle_rad", "<f8"), ("input_matches", "<i4"), ("landmark_count", "<i4"),
    ("cheirality_passes", "<i4"), ("pose_recovered", "<i4"),
])
assert TRI_RESULT_DTYPE.itemsize == 128


_vp = C.c_void_p
_ip = C.POINTER(C.c_int)
_u8pp = C.POINTER(C.POINTER(C.c_uint8))
_szp = C.POINTER(C.c_size_t)

# name -> (restype, argtypes)
SIGNATURES = {
    "uslam_create": (C.c_int, [C.POINTER(Params), C.POINTER(_vp)]),
    "uslam_destroy": (None, [_vp]),
    "uslam_last_error": (C.c_char_p, [_vp]),
    "uslam_status_string": (C.c_char_p, [C.c_int]),
    "uslam_level_dims": (C.c_int, [C.c_int, C.c_int, C.c_int, _ip, _ip]),
    "uslam_cull_coverage": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    "uslam_batch_create": (C.c_int, [_vp, C.c_int, _ip, _ip, C.c_int, _ip, _ip, C.POINTER(_vp)]),
    "uslam_batch_destroy": (None, [_vp]),
    "uslam_batch_input_device": (C.c_int, [_vp, C.c_int, _u8pp, _ip]),
    "uslam_batch_input_host": (C.c_int, [_vp, C.c_int, _u8pp, _ip]),
    "uslam_batch_set_frame": (C.c_int, [_vp, C.c_int, _vp, C.c_int]),
    "uslam_batch_upload": (C.c_int, [_vp]),
    "uslam_batch_run": (C.c_int, [_vp]),
    "uslam_batch_download": (C.c_int, [_vp]),
    "uslam_batch_sync": (C.c_int, [_vp, C.c_int]),
    "uslam_batch_features": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _ip, _ip]),
    "uslam_batch_matches": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _ip]),
    "uslam_batch_pyramid_level": (C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    "uslam_batch_keypoint_map": (C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    "uslam_batch_blur_level": (C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    "uslam_batch_set_stream": (C.c_int, [_vp, _vp]),
    "uslam_batch_profile": (C.c_int, [_vp, C.c_int, _vp]),
    "uslam_blur_margin": (C.c_int, [_vp, _ip]),
    "uslam_batch_set_first_wait": (C.c_int, [_vp, C.c_int, C.c_int]),
    "uslam_batch_io_bytes": (C.c_int, [_vp, _szp, _szp]),
    "uslam_tile_shapes": (C.c_int, [_ip, _ip, _ip]),
    "uslam_set_tile_shape": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int]),
    "uslam_get_tile_shape": (C.c_int, [_vp, C.c_int, C.c_int, _ip]),
    "uslam_autotune": (C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, C.c_int, _ip, _vp]),
    "uslam_frontend_create": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(_vp)]),
    "uslam_frontend_destroy": (None, [_vp]),
    "uslam_frontend_process": (C.c_int, [_vp, _vp, C.c_int, C.c_int]),
    "uslam_frontend_process_f32": (C.c_int, [_vp, _vp, C.c_int, C.c_int]),
    "uslam_frontend_input_device": (C.c_int, [_vp, _u8pp, _ip]),
    "uslam_frontend_features": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _ip, _ip]),
    "uslam_frontend_matches": (C.c_int, [_vp, _vp, C.c_int, _ip]),
    "uslam_frontend_enqueue": (C.c_int, [_vp, _vp, C.c_int, C.c_int, _ip]),
    "uslam_frontend_sync": (C.c_int, [_vp]),
    "uslam_server_create": (C.c_int, [_vp, C.POINTER(ServerParams), C.POINTER(_vp)]),
    "uslam_server_destroy": (None, [_vp]),
    "uslam_server_open_stream": (C.c_int, [_vp, C.c_int, C.c_int, _ip]),
    "uslam_server_submit": (C.c_int, [_vp, C.c_int, _vp, C.c_int, C.c_int, C.POINTER(C.c_uint64)]),
    "uslam_server_wait": (C.c_int, [_vp, C.c_uint64, C.c_int]),
    "uslam_server_result": (C.c_int, [_vp, C.c_uint64, _vp, C.c_int, _ip, _ip, _vp, C.c_int, _ip,
                                      C.POINTER(C.c_double)]),
    "uslam_server_release": (C.c_int, [_vp, C.c_uint64]),
    "uslam_server_stats": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), _ip, _ip]),
    "uslam_server_set_first_wait": (C.c_int, [_vp, C.c_int]),
    "uslam_featset_create": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(_vp)]),
    "uslam_featset_destroy": (None, [_vp]),
    "uslam_detect_describe": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    "uslam_detect_describe_f32": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    "uslam_featset_features": (C.c_int, [_vp, _vp, C.c_int, _ip, _ip]),
    "uslam_match_sets": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, _ip]),
    "uslam_ransac_score": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp, C.c_int, C.c_double, _ip, _vp]),
    "uslam_tri_default_opts": (None, [C.POINTER(TriOpts)]),
    "uslam_pixel_to_normalised": (C.c_int, [_vp, C.POINTER(Camera), C.c_int, C.c_double, _vp, C.c_int, _vp]),
    "uslam_triangulate": (C.c_int, [_vp, C.POINTER(Camera), C.POINTER(TriOpts), C.c_int, _ip, _vp, _vp, _vp, _vp]),
    "uslam_match_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _vp, _ip, _vp, _ip, _vp, _vp, C.c_int,
                                      _vp, C.c_char_p, C.c_size_t]),
}

_lib = None


def load(path: str | None = None):
    """Load libuslam.so and declare every exported signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with __graft_entry__.build() (no CPU fallback exists)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class USlamError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)
