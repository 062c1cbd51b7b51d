"""The reference's dataset reader (include/tsdfmc/dataset_io.h) over the portable native loader.

Layout: ``<root>/<frame id>/depth.png`` (grayscale PNG, raw x depth_scale = metres, 0 = invalid) and
``<root>/<frame id>/<pose file>`` (quaternion w x y z + translation, or a row-major 3x4 / 4x4 matrix); the
intrinsics metadata holds 5, 6 or 7 numbers (``fx fy cx cy [width height] [depth_scale]``) and falls back
to the first ``<root>/<frame>/params.txt``.  Same names, argument meanings and errors (RuntimeError where the
reference throws std::runtime_error) as the reference; the PNG decoding runs on any host, where the
reference's needs Windows WIC.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

from . import _capi
from .backend import DepthFrame
from .scenes import Intrinsics, Pose


def _check(status):
    if status != _capi.VH_OK:
        raise RuntimeError(_capi.lib().vh_dataset_last_error().decode(errors="replace"))


def _path(p) -> bytes:
    return os.fsencode(os.fspath(p))


@dataclasses.dataclass
class DatasetFrame:
    """dataset_io.h:30-35."""
    frame_id: int
    T_wc: Pose
    depth_frame: DepthFrame
    valid_depth_samples: int


def list_dataset_frame_ids(dataset_root) -> list[int]:
    """listDatasetFrameIds (dataset_io.h:135-152): all-digit subdirectory names, ascending."""
    n = C.c_size_t()
    _check(_capi.lib().vh_dataset_list_frames(_path(dataset_root), None, 0, C.byref(n)))
    ids = (C.c_int32 * max(1, n.value))()
    _check(_capi.lib().vh_dataset_list_frames(_path(dataset_root), ids, n.value, C.byref(n)))
    return [int(ids[i]) for i in range(n.value)]


def load_pose_from_file(path) -> Pose:
    """loadPoseFromFile (dataset_io.h:154-188)."""
    P = _capi.VhPose()
    _check(_capi.lib().vh_dataset_load_pose(_path(path), C.byref(P)))
    return Pose(np.array(P.R[:], np.float32).reshape(3, 3), np.array(P.t[:], np.float32))


def read_depth_png_gray16(path) -> np.ndarray:
    """The PNG as (H, W) uint16 gray (the WIC conversion of loadDepthPng, dataset_io.h:321-330)."""
    w, h = C.c_int32(), C.c_int32()
    _check(_capi.lib().vh_png_read_gray16(_path(path), None, 0, C.byref(w), C.byref(h)))
    out = np.zeros((h.value, w.value), np.uint16)
    _check(_capi.lib().vh_png_read_gray16(_path(path), out.ctypes.data_as(C.POINTER(C.c_uint16)), out.size,
                                          C.byref(w), C.byref(h)))
    return out


def load_depth_png(path, intrinsics: Intrinsics, depth_scale: float):
    """loadDepthPng (dataset_io.h:276-361): (DepthFrame, valid_depth_samples)."""
    K = _capi.intrinsics(intrinsics)
    depth = np.zeros((intrinsics.height, intrinsics.width), np.float32)
    valid = C.c_uint64()
    _check(_capi.lib().vh_dataset_load_depth_png(_path(path), C.byref(K), float(depth_scale),
                                                 depth.ctypes.data_as(C.POINTER(C.c_float)), C.byref(valid)))
    return DepthFrame(intrinsics, depth), int(valid.value)


def load_dataset_intrinsics(path):
    """loadDatasetIntrinsics (dataset_io.h:382-395): (Intrinsics, depth_scale)."""
    K = _capi.VhIntrinsics()
    scale = C.c_float()
    _check(_capi.lib().vh_dataset_load_intrinsics(_path(path), C.byref(K), C.byref(scale)))
    return Intrinsics(int(K.width), int(K.height), float(K.fx), float(K.fy), float(K.cx), float(K.cy)), float(scale.value)


def load_dataset_depth_frame(dataset_root, frame_id: int, pose_filename: str, intrinsics: Intrinsics,
                             depth_scale: float) -> DatasetFrame:
    """loadDatasetDepthFrame (dataset_io.h:397-409)."""
    frame_dir = os.path.join(os.fspath(dataset_root), str(frame_id))
    T = load_pose_from_file(os.path.join(frame_dir, pose_filename))
    frame, valid = load_depth_png(os.path.join(frame_dir, "depth.png"), intrinsics, depth_scale)
    return DatasetFrame(frame_id, T, frame, valid)
