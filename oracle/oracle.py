"""ctypes bindings for the parity oracle (oracle/liboracle.so) and, where it was built, the
reference itself (oracle/_ref/libref.so: the reference CPU path plus the reference CUDA kernels
run on the host under the emulation prelude).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg.  The product package never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

FLAVOR_REF_GPU = 0
FLAVOR_REF_CPU = 1
EXP_LIBM = 0
EXP_OWN = 1

VOXEL_DTYPE = np.dtype([("weight", "<f4"), ("surface_coord", "<f4"), ("plane_offset", "<f4"),
                        ("packed_normal", "<u4")])
VOXEL_BYTES = 6 * 3 * 16
BLOCK_VOXELS = 512


class VoConfig(C.Structure):
    _fields_ = [
        ("flavor", C.c_int32), ("exp_impl", C.c_int32),
        ("disc_base", C.c_float), ("disc_rel", C.c_float),
        ("filter_radius", C.c_int32), ("filter_sigma_spatial", C.c_float), ("filter_sigma_range", C.c_float),
        ("filter_sigma_angular", C.c_float), ("filter_min_cos", C.c_float),
        ("normal_radius", C.c_int32), ("normal_sigma_spatial", C.c_float), ("normal_sigma_range", C.c_float),
        ("normal_sigma_angular", C.c_float),
        ("layer_merge_scale", C.c_float), ("layer_normal_cos", C.c_float), ("layer_extract_scale", C.c_float),
        ("max_weight", C.c_float), ("depth_sigma", C.c_float), ("huber_delta", C.c_float),
        ("min_obs_weight", C.c_float), ("min_view_weight", C.c_float),
        ("threads", C.c_int32),
        ("alloc_mode", C.c_int32), ("normal_mode", C.c_int32), ("layer_format", C.c_int32),
    ]


class VoIntrinsics(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float)]


class VoPose(C.Structure):
    _fields_ = [("R", C.c_float * 9), ("t", C.c_float * 3)]


_lib = None
_lib64 = None
_ref = None

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_fp)


def lib(fp64=False):
    """The restatement (float arithmetic, bit-identical to the reference) or, with fp64, the FP64 transcription:
    the same source built with double arithmetic (oracle/liboracle64.so)."""
    global _lib, _lib64
    if fp64:
        if _lib64 is None:
            _lib64 = _load(os.path.join(HERE, "liboracle64.so"))
        return _lib64
    if _lib is None:
        _lib = _load(os.path.join(HERE, "liboracle.so"))
    return _lib


def _load(path):
    if not os.path.exists(path):
        from oracle import build as _b
        _b.build_oracle()
    L = C.CDLL(path)
    L.vo_config_default.argtypes = [C.POINTER(VoConfig), C.c_int32]
    L.vo_expf_own.argtypes = [C.c_float]
    L.vo_expf_own.restype = C.c_float
    L.vo_expf_array.argtypes = [_fp, _fp, C.c_size_t]
    L.vo_render_depth.argtypes = [_fp, C.c_int32, C.POINTER(VoIntrinsics), C.POINTER(VoPose), C.c_uint32, C.c_uint32,
                                  C.c_float, C.c_float, C.c_float, _fp]
    L.vo_expf_compare_libm.argtypes = [C.c_uint32, C.c_uint64, C.c_int, C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_uint32)]
    L.vo_filter_depth.argtypes = [C.POINTER(VoConfig), _fp, C.POINTER(VoIntrinsics), _fp]
    L.vo_depth_normals.argtypes = [C.POINTER(VoConfig), _fp, C.POINTER(VoIntrinsics), _fp,
                                   C.POINTER(C.c_uint8)]
    L.vo_raycast_depth.argtypes = [C.c_void_p, C.POINTER(VoIntrinsics), C.POINTER(VoPose), C.c_float, C.c_float,
                                   C.c_float, _fp]
    L.vo_surface_normal.argtypes = [C.POINTER(VoConfig), _fp, C.POINTER(VoIntrinsics), C.c_float, C.c_float,
                                    _fp]
    L.vo_surface_normal.restype = C.c_int32
    L.vo_collect_blocks.argtypes = [C.POINTER(VoConfig), _fp, C.POINTER(VoIntrinsics), C.POINTER(VoPose),
                                    C.c_float, C.c_float, C.c_int32, _ip, C.c_int64]
    L.vo_collect_blocks.restype = C.c_int64
    L.vo_collect_band_blocks.argtypes = [_fp, C.POINTER(VoIntrinsics), C.POINTER(VoPose), C.c_float, C.c_float,
                                         C.c_int32, _ip, C.c_int64]
    L.vo_collect_band_blocks.restype = C.c_int64
    L.vo_volume_new.argtypes = [C.POINTER(VoConfig), C.c_float, C.c_float]
    L.vo_volume_new.restype = C.c_void_p
    L.vo_volume_free.argtypes = [C.c_void_p]
    L.vo_volume_integrate_frame.argtypes = [C.c_void_p, _fp, C.POINTER(VoIntrinsics), C.POINTER(VoPose),
                                            C.c_int32]
    L.vo_volume_integrate_frame.restype = C.c_int64
    L.vo_volume_integrate_blocks.argtypes = [C.c_void_p, _ip, C.c_int64, _fp, C.POINTER(VoIntrinsics),
                                             C.POINTER(VoPose)]
    L.vo_volume_block_count.argtypes = [C.c_void_p]
    L.vo_volume_block_count.restype = C.c_int64
    L.vo_volume_observed_voxels.argtypes = [C.c_void_p]
    L.vo_volume_observed_voxels.restype = C.c_int64
    L.vo_volume_get_block.argtypes = [C.c_void_p, C.c_int64, _ip, C.c_void_p]
    L.vo_volume_find_block.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
    L.vo_volume_find_block.restype = C.c_int64
    L.vo_volume_set_block.argtypes = [C.c_void_p, C.c_int32 * 3, C.c_void_p]
    L.vo_volume_apply_flat_blocks.argtypes = [C.c_void_p, _ip, C.c_void_p, C.c_int64]
    L.vo_volume_remove_blocks.argtypes = [C.c_void_p, _ip, C.c_int64]
    L.vo_volume_extract_mesh.argtypes = [C.c_void_p, C.c_float, C.POINTER(C.c_void_p)]
    L.vo_volume_extract_mesh.restype = C.c_int64
    L.vo_free.argtypes = [C.c_void_p]
    L.vo_pack_normal.argtypes = [C.c_int32, _fp]
    L.vo_pack_normal.restype = C.c_uint32
    L.vo_unpack_normal.argtypes = [C.c_int32, C.c_int32, C.c_uint32, _fp]
    L.vo_hash_block_key.argtypes = [C.c_int32, C.c_int32, C.c_int32]
    L.vo_hash_block_key.restype = C.c_uint32
    L.vo_pack_block_key.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_uint64)]
    L.vo_pack_block_key.restype = C.c_int32
    L.vo_observation_weight.argtypes = [C.POINTER(VoConfig), C.c_float, C.c_float, C.c_float, C.c_float]
    L.vo_observation_weight.restype = C.c_float
    return L


def config(flavor=FLAVOR_REF_GPU, exp_impl=EXP_OWN, threads=1, **overrides) -> VoConfig:
    c = VoConfig()
    lib().vo_config_default(C.byref(c), flavor)
    c.exp_impl = exp_impl
    c.threads = threads
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def intrinsics(K) -> VoIntrinsics:
    return VoIntrinsics(int(K.width), int(K.height), float(K.fx), float(K.fy), float(K.cx), float(K.cy))


def pose(P) -> VoPose:
    p = VoPose()
    p12 = P.as12() if hasattr(P, "as12") else np.asarray(P, np.float32).reshape(12)
    for i in range(9):
        p.R[i] = float(p12[i])
    for i in range(3):
        p.t[i] = float(p12[9 + i])
    return p


def expf_own(x: float) -> float:
    return lib().vo_expf_own(x)


def render_depth(scene, frame, noise=True):
    """The device renderer's frame (vh_render_depth), restated on the host: bit-identical float32 HxW depth."""
    K = scene.intrinsics
    prims = np.ascontiguousarray(scene.prims, np.float32)
    out = np.empty((K.height, K.width), np.float32)
    Ki, Pi = intrinsics(K), pose(scene.poses[frame])
    lib().vo_render_depth(prims.ctypes.data_as(_fp), prims.shape[0], C.byref(Ki), C.byref(Pi), scene.seed, frame,
                          scene.noise_sigma_z2 if noise else 0.0, scene.dropout if noise else 0.0, scene.max_depth,
                          out.ctypes.data_as(_fp))
    return out


def expf_array(x):
    """vo_expf_own element-wise over a float32 array."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    lib().vo_expf_array(x.ctypes.data_as(_fp), y.ctypes.data_as(_fp), x.size)
    return y


def expf_compare_libm(first_bits, count, threads=8):
    """(mismatches, smallest mismatching bit pattern or 0xffffffff) of vo_expf_own vs the C library's expf over the
    float bit patterns [first_bits, first_bits + count), NaNs excluded."""
    n, f = C.c_uint64(), C.c_uint32()
    lib().vo_expf_compare_libm(first_bits, count, threads, C.byref(n), C.byref(f))
    return n.value, f.value


def filter_depth(cfg, depth, K, fp64=False):
    d, dp = _f32(depth)
    out = np.zeros_like(d)
    lib(fp64).vo_filter_depth(C.byref(cfg), dp, C.byref(intrinsics(K)), out.ctypes.data_as(_fp))
    return out


def depth_normals(cfg, depth, K, fp64=False):
    d, dp = _f32(depth)
    n = np.zeros(d.shape + (3,), np.float32)
    v = np.zeros(d.shape, np.uint8)
    lib(fp64).vo_depth_normals(C.byref(cfg), dp, C.byref(intrinsics(K)), n.ctypes.data_as(_fp),
                               v.ctypes.data_as(C.POINTER(C.c_uint8)))
    return n, v


def pixel_normals(cfg, depth, K):
    """estimateSurfaceNormalCamera at every pixel centre: normals (H, W, 3) float32, valid (H, W) uint8."""
    d, dp = _f32(depth)
    n = np.zeros(d.shape + (3,), np.float32)
    ok = np.zeros(d.shape, np.uint8)
    out = np.zeros(3, np.float32)
    Ki = intrinsics(K)
    for y in range(d.shape[0]):
        for x in range(d.shape[1]):
            if lib().vo_surface_normal(C.byref(cfg), dp, C.byref(Ki), float(x), float(y), out.ctypes.data_as(_fp)):
                ok[y, x] = 1
                n[y, x] = out
    return n, ok


def collect_blocks(cfg, depth, K, P, voxel_size, truncation, stride=1, fp64=False):
    d, dp = _f32(depth)
    cap = max(1024, int(d.size) * 81 // max(1, stride * stride) + 1024)
    keys = np.zeros((cap, 3), np.int32)
    n = lib(fp64).vo_collect_blocks(C.byref(cfg), dp, C.byref(intrinsics(K)), C.byref(pose(P)), voxel_size,
                                truncation, stride, keys.ctypes.data_as(_ip), cap)
    if n < 0:
        return None
    return keys[:n].copy()


def collect_band_blocks(depth, K, P, voxel_size, truncation, stride=1):
    """Keys of the truncation-band rule (the library's opt-in allocation mode), sorted; None on key overflow."""
    d, dp = _f32(depth)
    cap = max(1024, int(d.size) * 64 // max(1, stride * stride) + 1024)
    keys = np.zeros((cap, 3), np.int32)
    n = lib().vo_collect_band_blocks(dp, C.byref(intrinsics(K)), C.byref(pose(P)), voxel_size, truncation, stride,
                                     keys.ctypes.data_as(_ip), cap)
    if n < 0:
        return None
    return keys[:n].copy()


class Volume:
    """The oracle's voxel-hash volume (reference layout: 12-byte key + 512 x 288-byte voxels)."""

    def __init__(self, cfg, voxel_size, truncation, fp64=False):
        """fp64: the FP64 transcription's volume (double arithmetic, float voxel records)."""
        self.cfg = cfg
        self.L = lib(fp64)
        self.h = self.L.vo_volume_new(C.byref(cfg), voxel_size, truncation)

    def close(self):
        if self.h:
            self.L.vo_volume_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def integrate(self, depth, K, P, stride=1):
        d, dp = _f32(depth)
        return self.L.vo_volume_integrate_frame(self.h, dp, C.byref(intrinsics(K)), C.byref(pose(P)), stride)

    def integrate_blocks(self, keys, depth, K, P):
        k = np.ascontiguousarray(keys, np.int32).reshape(-1, 3)
        d, dp = _f32(depth)
        self.L.vo_volume_integrate_blocks(self.h, k.ctypes.data_as(_ip), k.shape[0], dp, C.byref(intrinsics(K)),
                                         C.byref(pose(P)))

    def raycast_depth(self, K, P, min_depth=0.1, max_depth=8.0, step_voxels=0.5):
        """Depth (H, W) float32 of the product's ray-cast definition on this volume; 0 = no hit."""
        out = np.zeros((K.height, K.width), np.float32)
        self.L.vo_raycast_depth(self.h, C.byref(intrinsics(K)), C.byref(pose(P)), float(min_depth), float(max_depth),
                               float(step_voxels), out.ctypes.data_as(_fp))
        return out

    def block_count(self):
        return self.L.vo_volume_block_count(self.h)

    def observed_voxels(self):
        return self.L.vo_volume_observed_voxels(self.h)

    def blocks(self):
        """(keys (N,3) int32, voxels (N,512,6,3) structured VOXEL_DTYPE) in insertion order."""
        n = self.block_count()
        keys = np.zeros((n, 3), np.int32)
        vox = np.zeros((n, BLOCK_VOXELS, 6, 3), VOXEL_DTYPE)
        for i in range(n):
            self.L.vo_volume_get_block(self.h, i, keys[i].ctypes.data_as(_ip), vox[i].ctypes.data)
        return keys, vox

    def set_block(self, key, voxels):
        v = np.ascontiguousarray(voxels, VOXEL_DTYPE)
        self.L.vo_volume_set_block(self.h, (C.c_int32 * 3)(*map(int, key)), v.ctypes.data)

    def apply_flat_blocks(self, keys, voxels):
        """applyFlatBlocks (voxel_hash_tsdf.h:183-188): keys (N,3) int32, voxels (N,512,6,3) VOXEL_DTYPE or the
        same bytes as a flat array, applied in order."""
        k = np.ascontiguousarray(keys, np.int32).reshape(-1, 3)
        v = np.ascontiguousarray(voxels).view(np.uint8).reshape(k.shape[0], -1)
        assert v.shape[1] == BLOCK_VOXELS * VOXEL_BYTES
        self.L.vo_volume_apply_flat_blocks(self.h, k.ctypes.data_as(_ip), v.ctypes.data, k.shape[0])

    def remove_blocks(self, keys):
        """The library's eviction of these blocks (no reference counterpart)."""
        k = np.ascontiguousarray(keys, np.int32).reshape(-1, 3)
        self.L.vo_volume_remove_blocks(self.h, k.ctypes.data_as(_ip), k.shape[0])

    def extract_mesh(self, iso=0.0):
        ptr = C.c_void_p()
        n = self.L.vo_volume_extract_mesh(self.h, iso, C.byref(ptr))
        if n == 0:
            self.L.vo_free(ptr)
            return np.zeros((0, 9), np.float32)
        arr = np.ctypeslib.as_array(C.cast(ptr, _fp), shape=(n * 9,)).reshape(n, 9).copy()
        self.L.vo_free(ptr)
        return arr


# ------------------------------------------------------------------ reference (x86 build host only)
def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libref.so"))


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(os.path.join(HERE, "_ref", "libref.so"))
        R.ref_cpu_filter.argtypes = [_fp, C.c_int, C.c_int, _fp, _fp]
        R.ref_gpu_filter.argtypes = [_fp, C.c_int, C.c_int, _fp, _fp, _fp, C.POINTER(C.c_uint8)]
        for name in ("ref_cpu_collect", "ref_gpu_allocate"):
            f = getattr(R, name)
            f.argtypes = [_fp, C.c_int, C.c_int, _fp, _fp, C.c_float, C.c_float, C.c_int, _ip, C.c_long]
            f.restype = C.c_long
        R.ref_new.argtypes = [C.c_int, C.c_float, C.c_float]
        R.ref_new.restype = C.c_void_p
        R.ref_free.argtypes = [C.c_void_p]
        R.ref_integrate.argtypes = [C.c_void_p, _fp, C.c_int, C.c_int, _fp, _fp, C.c_int]
        R.ref_block_count.argtypes = [C.c_void_p]
        R.ref_block_count.restype = C.c_long
        R.ref_observed.argtypes = [C.c_void_p]
        R.ref_observed.restype = C.c_long
        R.ref_extract.argtypes = [C.c_void_p, C.c_float]
        R.ref_extract.restype = C.c_long
        R.ref_mesh_copy.argtypes = [C.c_void_p, _fp]
        R.ref_get_blocks.argtypes = [C.c_void_p, _ip, C.c_void_p, C.c_long]
        R.ref_get_blocks.restype = C.c_long
        R.ref_cpu_pack_normal.argtypes = [_fp]
        R.ref_cpu_pack_normal.restype = C.c_uint
        R.ref_cpu_unpack_normal.argtypes = [C.c_uint, _fp]
        R.ref_gpu_pack_normal.argtypes = [_fp]
        R.ref_gpu_pack_normal.restype = C.c_uint
        R.ref_gpu_unpack_normal.argtypes = [C.c_uint, _fp]
        R.ref_gpu_mesh_unpack_normal.argtypes = [C.c_uint, _fp]
        R.ref_gpu_hash_block_key.argtypes = [C.c_int, C.c_int, C.c_int]
        R.ref_gpu_hash_block_key.restype = C.c_uint
        R.ref_gpu_pack_block_key.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_ulonglong)]
        R.ref_gpu_pack_block_key.restype = C.c_int
        R.ref_gpu_observation_weight.argtypes = [C.c_float] * 4
        R.ref_gpu_observation_weight.restype = C.c_float
        _ref = R
    return _ref


def ref_filter(depth, K, gpu: bool):
    d, dp = _f32(depth)
    out = np.zeros_like(d)
    k4, k4p = _f32(K.k4())
    if gpu:
        ref().ref_gpu_filter(dp, K.width, K.height, k4p, out.ctypes.data_as(_fp), None, None)
    else:
        ref().ref_cpu_filter(dp, K.width, K.height, k4p, out.ctypes.data_as(_fp))
    return out


def ref_collect(depth, K, P, voxel_size, truncation, stride, gpu: bool):
    d, dp = _f32(depth)
    k4, k4p = _f32(K.k4())
    p12, pp = _f32(P.as12())
    cap = max(1024, int(d.size) * 81 + 1024)
    keys = np.zeros((cap, 3), np.int32)
    fn = ref().ref_gpu_allocate if gpu else ref().ref_cpu_collect
    n = fn(dp, K.width, K.height, k4p, pp, voxel_size, truncation, stride, keys.ctypes.data_as(_ip), cap)
    if n < 0:
        return None
    k = keys[:n]
    return k[np.lexsort((k[:, 2], k[:, 1], k[:, 0]))].copy()


class RefVolume:
    """The reference backend (TsdfIntegrationBackend + VoxelHashTSDF), CPU or emulated GPU path."""

    def __init__(self, gpu: bool, voxel_size, truncation):
        self.h = ref().ref_new(1 if gpu else 0, voxel_size, truncation)

    def close(self):
        if self.h:
            ref().ref_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def integrate(self, depth, K, P, stride=1):
        d, dp = _f32(depth)
        k4, k4p = _f32(K.k4())
        p12, pp = _f32(P.as12())
        ref().ref_integrate(self.h, dp, K.width, K.height, k4p, pp, stride)

    def block_count(self):
        return ref().ref_block_count(self.h)

    def observed_voxels(self):
        return ref().ref_observed(self.h)

    def extract_mesh(self, iso=0.0):
        n = ref().ref_extract(self.h, iso)
        out = np.zeros((n, 9), np.float32)
        if n:
            ref().ref_mesh_copy(self.h, out.ctypes.data_as(_fp))
        return out

    def blocks(self):
        n = self.block_count()
        keys = np.zeros((n, 3), np.int32)
        vox = np.zeros((n, BLOCK_VOXELS, 6, 3), VOXEL_DTYPE)
        got = ref().ref_get_blocks(self.h, keys.ctypes.data_as(_ip), vox.ctypes.data, n)
        assert got == n, (got, n)
        return keys, vox


# ------------------------------------------------------------------ comparison helpers
def sort_blocks(keys, vox):
    order = np.lexsort((keys[:, 2], keys[:, 1], keys[:, 0]))
    return keys[order], vox[order]


def canonical_triangles(tris):
    """Triangles as a lexicographically sorted (N,9) float32 array (multiset comparison)."""
    t = np.asarray(tris, np.float32).reshape(-1, 9)
    if t.shape[0] == 0:
        return t
    bits = t.view(np.uint32)
    order = np.lexsort(tuple(bits[:, i] for i in range(8, -1, -1)))
    return t[order]
