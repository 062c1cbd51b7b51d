"""ctypes binding of the C ABI in include/voxelhash_gb300.h (libvoxelhash_gb300.so, built in-tree).

The library is the product: there is no fallback.  ``lib()`` raises if the shared library has not been
built (``python -m voxelhashmt_gb300.build``), and every call that
returns a non-zero vh_status raises ``VhError`` carrying the status and the volume's last error message.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libvoxelhash_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "voxelhash_gb300.h")

VH_OK = 0
VH_ERR_INVALID_ARGUMENT = 1
VH_ERR_CUDA = 2
VH_ERR_NO_DEVICE = 3
VH_ERR_OUT_OF_MEMORY = 4
VH_ERR_KEY_RANGE = 5
VH_ERR_HASH_FULL = 6
VH_ERR_POOL_FULL = 7
VH_ERR_BUFFER_TOO_SMALL = 8
VH_ERR_CAPACITY = 9
VH_ERR_IO = 10
VH_ERR_FORMAT = 11
VH_ERR_TIMEOUT = 12

BLOCK_BYTES = 512 * 6 * 3 * 16


class VhParams(C.Structure):
    _fields_ = [("voxel_size", C.c_float), ("truncation_distance", C.c_float), ("hash_buckets", C.c_uint32),
                ("max_blocks", C.c_uint32), ("device", C.c_int32), ("layer_format", C.c_int32)]


class VhAlgorithm(C.Structure):
    _fields_ = [
        ("depth_discontinuity_base", C.c_float), ("depth_discontinuity_relative", C.c_float),
        ("filter_radius", C.c_int32), ("filter_sigma_spatial", C.c_float), ("filter_sigma_range", C.c_float),
        ("filter_sigma_angular", C.c_float), ("filter_min_cosine", C.c_float),
        ("normal_radius", C.c_int32), ("normal_sigma_spatial", C.c_float), ("normal_sigma_range", C.c_float),
        ("normal_sigma_angular", C.c_float),
        ("layer_merge_voxel_scale", C.c_float), ("layer_normal_cosine", C.c_float),
        ("layer_extract_voxel_scale", C.c_float),
        ("max_voxel_weight", C.c_float), ("depth_sigma", C.c_float), ("huber_delta", C.c_float),
        ("min_observation_weight", C.c_float), ("min_view_angle_weight", C.c_float),
        ("allocation_mode", C.c_int32), ("fast_math", C.c_int32), ("normal_mode", C.c_int32),
        ("autotune", C.c_int32), ("launch_variant", C.c_int32), ("depth_filter", C.c_int32),
    ]


class VhIntrinsics(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float)]


class VhPose(C.Structure):
    _fields_ = [("R", C.c_float * 9), ("t", C.c_float * 3)]


class VhFrameStats(C.Structure):
    _fields_ = [("visible_blocks", C.c_uint64), ("new_blocks", C.c_uint64), ("active_voxels", C.c_uint64),
                ("updated_voxels", C.c_uint64),
                ("total_blocks", C.c_uint64), ("observed_voxels", C.c_uint64)]


class VhError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (_status_name(status), status, message))
        self.status = status


def _status_name(status):
    names = {0: "VH_OK", 1: "VH_ERR_INVALID_ARGUMENT", 2: "VH_ERR_CUDA", 3: "VH_ERR_NO_DEVICE",
             4: "VH_ERR_OUT_OF_MEMORY", 5: "VH_ERR_KEY_RANGE", 6: "VH_ERR_HASH_FULL", 7: "VH_ERR_POOL_FULL",
             8: "VH_ERR_BUFFER_TOO_SMALL", 9: "VH_ERR_CAPACITY", 10: "VH_ERR_IO", 11: "VH_ERR_FORMAT", 12: "VH_ERR_TIMEOUT"}
    return names.get(status, "VH_STATUS_%d" % status)


_lib = None
_vp = C.c_void_p
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_u64p = C.POINTER(C.c_uint64)
_szp = C.POINTER(C.c_size_t)

_SIGNATURES = {
    "vh_params_default": (None, [C.POINTER(VhParams)]),
    "vh_algorithm_default": (None, [C.POINTER(VhAlgorithm)]),
    "vh_status_string": (C.c_char_p, [C.c_int]),
    "vh_query_device": (C.c_int, [C.c_char_p, C.c_size_t]),
    "vh_create": (C.c_int, [C.POINTER(VhParams), C.POINTER(VhAlgorithm), C.POINTER(_vp)]),
    "vh_destroy": (None, [_vp]),
    "vh_reset": (C.c_int, [_vp, _vp]),
    "vh_last_error": (C.c_char_p, [_vp]),
    "vh_integrate": (C.c_int, [_vp, _vp, C.c_int32, C.POINTER(VhIntrinsics), C.POINTER(VhPose), C.c_int32, _vp]),
    "vh_allocate": (C.c_int, [_vp, _vp, C.c_int32, C.POINTER(VhIntrinsics), C.POINTER(VhPose), C.c_int32, _ip,
                              C.c_size_t, _szp, _vp]),
    "vh_visible_block_keys": (C.c_int, [_vp, _ip, C.c_size_t, _szp, _vp]),
    "vh_filter_depth": (C.c_int, [_vp, _vp, _vp, C.POINTER(VhIntrinsics), _vp]),
    "vh_depth_normals": (C.c_int, [_vp, _vp, _vp, _vp, C.POINTER(VhIntrinsics), _vp]),
    "vh_pixel_normals": (C.c_int, [_vp, _vp, _vp, C.POINTER(VhIntrinsics), _vp]),
    "vh_raycast_depth": (C.c_int, [_vp, C.POINTER(VhIntrinsics), C.POINTER(VhPose), C.c_float, C.c_float, C.c_float,
                                   _vp, _vp]),
    "vh_synchronize": (C.c_int, [_vp, _vp]),
    "vh_extract_mesh": (C.c_int, [_vp, C.c_float, _szp, _vp]),
    "vh_extract_mesh_recent": (C.c_int, [_vp, C.c_float, C.c_uint32, _szp, _vp]),
    "vh_frame_stats_enqueue": (C.c_int, [_vp, _vp, _vp]),
    "vh_frame_stats_decode": (C.c_int, [_vp, _vp, C.POINTER(VhFrameStats)]),
    "vh_copy_mesh": (C.c_int, [_vp, _vp, C.c_size_t, C.c_int32, _vp]),
    "vh_weld_mesh": (C.c_int, [_vp, _szp, _szp, _vp]),
    "vh_copy_welded_mesh": (C.c_int, [_vp, _vp, C.c_size_t, _vp, C.c_size_t, C.c_int32, _vp]),
    "vh_block_count": (C.c_int, [_vp, _u64p]),
    "vh_observed_voxel_count": (C.c_int, [_vp, _u64p]),
    "vh_recount_observed_voxels": (C.c_int, [_vp, _u64p, _vp]),
    "vh_frame_stats_get": (C.c_int, [_vp, C.POINTER(VhFrameStats), _vp]),
    "vh_export_blocks": (C.c_int, [_vp, C.c_uint64, C.c_uint64, _ip, _vp, C.c_int32, _vp]),
    "vh_allocate_static_scratch": (C.c_int, [_vp, C.POINTER(VhIntrinsics), C.POINTER(VhPose), C.c_float, C.c_float,
                                             C.c_int32, _vp, C.c_size_t, _szp, _vp]),
    "vh_import_blocks": (C.c_int, [_vp, _ip, _vp, C.c_uint64, C.c_int32, _vp]),
    "vh_autotune_result": (C.c_int, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_float)]),
    "vh_profile_enable": (C.c_int, [_vp, C.c_int32]),
    "vh_batch_create": (C.c_int, [C.POINTER(_vp), C.c_int32, C.c_int32, C.POINTER(_vp)]),
    "vh_batch_destroy": (None, [_vp]),
    "vh_batch_integrate": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(VhIntrinsics), C.POINTER(VhPose), _ip, C.c_int32,
                                     _vp]),
    "vh_nn_pack_conv32_weights": (C.c_int, [_vp, _vp, C.c_int32, _vp]),
    "vh_nn_conv32": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                               C.POINTER(C.c_uint32), _vp]),
    "vh_nn_conv32_gated": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                     C.c_int32, _vp, C.POINTER(C.c_uint32), _vp]),
    "vh_nn_wgrad32": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_uint32), _vp]),
    "vh_nn_param_count": (C.c_int32, []),
    "vh_nn_workspace_bytes": (C.c_uint64, [C.c_int32, C.c_int32, C.c_int32]),
    "vh_nn_pack": (C.c_int, [_vp, _vp, _vp]),
    "vh_nn_forward": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, _vp, C.POINTER(C.c_uint32), _vp]),
    "vh_nn_backward": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, _vp, _vp, _vp,
                                 C.POINTER(C.c_uint32), _vp]),
    "vh_nn_adam": (C.c_int, [_vp, _vp, _vp, _vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32, _vp]),
    "vh_set_depth_denoiser": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "vh_dataset_last_error": (C.c_char_p, []),
    "vh_dataset_list_frames": (C.c_int, [C.c_char_p, _ip, C.c_size_t, _szp]),
    "vh_dataset_load_intrinsics": (C.c_int, [C.c_char_p, C.POINTER(VhIntrinsics), C.POINTER(C.c_float)]),
    "vh_dataset_load_pose": (C.c_int, [C.c_char_p, C.POINTER(VhPose)]),
    "vh_png_read_gray16": (C.c_int, [C.c_char_p, C.POINTER(C.c_uint16), C.c_size_t, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
    "vh_dataset_load_depth_png": (C.c_int, [C.c_char_p, C.POINTER(VhIntrinsics), C.c_float, C.POINTER(C.c_float),
                                            _u64p]),
    "vh_profile_read": (C.c_int, [_vp, C.POINTER(C.c_double), _u64p]),
    "vh_render_depth": (C.c_int, [_vp, C.c_int32, C.POINTER(VhIntrinsics), C.POINTER(VhPose), C.c_uint32,
                                  C.c_uint32, C.c_float, C.c_float, C.c_float, _vp, _vp]),
    "vh_expf_eval": (C.c_int, [_vp, _vp, C.c_uint64, _vp]),
    "vh_evict_blocks": (C.c_int, [_vp, C.c_uint32, C.c_uint64, C.c_int32, _vp, _vp, C.c_uint64, C.c_int32, _u64p,
                                  _vp]),
    "vh_restore_blocks": (C.c_int, [_vp, _vp, _vp, C.c_uint64, C.c_int32, _vp]),
    "vh_expf_check": (C.c_int, [C.c_uint32, C.c_uint64, _u64p, C.POINTER(C.c_uint32), _vp]),
}


def header_symbols():
    """Every function the public header declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(vh_\w+)\s*\(", text, flags=re.M)))


def lib():
    """The loaded CUDA library; raises if it was not built (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libvoxelhash_gb300.so is not built (%s); run python -m voxelhashmt_gb300.build" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status, handle=None):
    if status != VH_OK:
        msg = ""
        if handle:
            msg = lib().vh_last_error(handle).decode(errors="replace")
        if not msg:
            msg = lib().vh_status_string(status).decode()
        raise VhError(status, msg)
    return status


def default_params(**kw) -> VhParams:
    p = VhParams()
    lib().vh_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def default_algorithm(**kw) -> VhAlgorithm:
    a = VhAlgorithm()
    lib().vh_algorithm_default(C.byref(a))
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def intrinsics(K) -> VhIntrinsics:
    return VhIntrinsics(int(K.width), int(K.height), float(K.fx), float(K.fy), float(K.cx), float(K.cy))


def pose(P) -> VhPose:
    import numpy as np
    p12 = P.as12() if hasattr(P, "as12") else np.asarray(P, np.float32).reshape(12)
    out = VhPose()
    for i in range(9):
        out.R[i] = float(p12[i])
    for i in range(3):
        out.t[i] = float(p12[9 + i])
    return out
