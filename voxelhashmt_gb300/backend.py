"""Host-side mirror of the reference's reconstruction backend over the GB300 C ABI.

Mirrors (paths relative to the reference project):
  TsdfIntegrationBackend             include/tsdfmc/reconstruction_backend.h:18-42
  ComputeBackendPreference / parse   include/tsdfmc/reconstruction_backend.h:9-16
  VoxelHashTSDF (device-resident)    include/tsdfmc/voxel_hash_tsdf.h:53-188 (the state the reference keeps in
                                     its GpuVolumeCache singleton, src/cuda_tsdf_integrator.cu:114-167)
  allocate_active_blocks_cuda        src/cuda_block_allocator.h:17-22
  integrate_depth_frame_cuda         src/cuda_tsdf_integrator.h:16-19
  extract_mesh_cuda                  src/cuda_mesh_extractor.h:9
  query_cuda_backend_status / gpu_volume_cache_*   src/cuda_tsdf_integrator.h:9-25

Differences that follow from the GB300 design: there is no CPU backend and no fallback (a CPU
preference raises, as the reference's kGpu does without CUDA); the volume owns its device state (no
process-wide singleton bound to one volume at a time); allocation overflow raises VhError instead of
silently switching to the CPU allocator.  Depth may be a numpy array (host) or a contiguous float32
CUDA tensor (device); ``stream`` is a torch.cuda.Stream, a raw cudaStream_t integer, or None.
"""
from __future__ import annotations

import ctypes as C
import enum

import numpy as np

from . import _capi
from .scenes import Intrinsics, Pose  # noqa: F401  (re-exported: math_types.h equivalents)


class ComputeBackendPreference(enum.Enum):
    AUTO = "auto"
    CPU = "cpu"
    GPU = "gpu"


def parse_compute_backend_preference(value: str) -> ComputeBackendPreference:
    """reconstruction_backend.cpp:205-220 (case-insensitive auto|cpu|gpu); raises ValueError otherwise."""
    try:
        return ComputeBackendPreference(value.lower())
    except ValueError:
        raise ValueError("invalid backend preference %r (expected auto|cpu|gpu)" % value) from None


def query_cuda_backend_status():
    """(runtime_available, message) -- queryCudaBackendStatus, cuda_tsdf_integrator.cu:934-944."""
    buf = C.create_string_buffer(256)
    st = _capi.lib().vh_query_device(buf, len(buf))
    return st == _capi.VH_OK, buf.value.decode()


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


class DepthFrame:
    """math_types.h:209-226: intrinsics + row-major float32 depth (metres, <= 0 invalid)."""

    def __init__(self, intrinsics, depth):
        self.intrinsics = intrinsics
        self.depth = depth

    def _pointer(self):
        d = self.depth
        if hasattr(d, "is_cuda") and d.is_cuda:
            if d.dtype.__repr__() != "torch.float32" or not d.is_contiguous():
                raise ValueError("device depth must be a contiguous float32 tensor")
            if d.numel() != self.intrinsics.width * self.intrinsics.height:
                raise ValueError("depth size does not match the intrinsics")
            return C.c_void_p(d.data_ptr()), 1, d
        a = np.ascontiguousarray(np.asarray(d, dtype=np.float32))
        if a.size != self.intrinsics.width * self.intrinsics.height:
            raise ValueError("depth size does not match the intrinsics")
        return C.c_void_p(a.ctypes.data), 0, a


class VoxelHashTSDF:
    """A voxel-hashed directional multi-layer volume resident on one GPU."""

    def __init__(self, voxel_size, truncation_distance, hash_buckets=1 << 16, max_blocks=1 << 14, device=0,
                 algorithm: _capi.VhAlgorithm | None = None, layer_format=0):
        """layer_format 0: FP32 layer records (the reference's); 1: FP16 storage (weight, and surface
        coordinate / plane offset relative to the voxel centre, in binary16) with FP32 update arithmetic."""
        self._voxel_size = float(voxel_size)
        self._truncation = float(truncation_distance)
        params = _capi.default_params(voxel_size=self._voxel_size, truncation_distance=self._truncation,
                                      hash_buckets=int(hash_buckets), max_blocks=int(max_blocks), device=int(device),
                                      layer_format=int(layer_format))
        self.algorithm = algorithm if algorithm is not None else _capi.default_algorithm()
        h = C.c_void_p()
        _capi.check(_capi.lib().vh_create(C.byref(params), C.byref(self.algorithm), C.byref(h)))
        self.handle = h
        self.max_blocks = int(max_blocks)
        self.hash_buckets = int(hash_buckets)
        self.layer_format = int(layer_format)
        self.device = int(device)

    def close(self):
        if getattr(self, "handle", None):
            _capi.lib().vh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def voxel_size(self):
        return self._voxel_size

    def truncation_distance(self):
        return self._truncation

    def reset(self, stream=None):
        _capi.check(_capi.lib().vh_reset(self.handle, _stream_handle(stream)), self.handle)

    def synchronize(self, stream=None):
        _capi.check(_capi.lib().vh_synchronize(self.handle, _stream_handle(stream)), self.handle)

    def block_count(self):
        n = C.c_uint64()
        _capi.check(_capi.lib().vh_block_count(self.handle, C.byref(n)), self.handle)
        return n.value

    def observed_voxel_count(self):
        n = C.c_uint64()
        _capi.check(_capi.lib().vh_observed_voxel_count(self.handle, C.byref(n)), self.handle)
        return n.value

    def recount_observed_voxels(self, stream=None):
        n = C.c_uint64()
        _capi.check(_capi.lib().vh_recount_observed_voxels(self.handle, C.byref(n), _stream_handle(stream)),
                    self.handle)
        return n.value

    def frame_stats(self, stream=None):
        s = _capi.VhFrameStats()
        _capi.check(_capi.lib().vh_frame_stats_get(self.handle, C.byref(s), _stream_handle(stream)), self.handle)
        return {f: getattr(s, f) for f, _ in s._fields_}

    def autotune_result(self):
        """{'variant', 'threads_per_cta', 'min_ctas_per_sm', 'ms'} of the layer-update launch shape the
        autotuner kept (variant -1 while tuning)."""
        v, t, b = C.c_int32(), C.c_int32(), C.c_int32()
        ms = C.c_float()
        _capi.check(_capi.lib().vh_autotune_result(self.handle, C.byref(v), C.byref(t), C.byref(b), C.byref(ms)),
                    self.handle)
        return {"variant": v.value, "threads_per_cta": t.value, "min_ctas_per_sm": b.value, "ms": ms.value}

    def frame_stats_enqueue(self, counters64, stream=None):
        """Enqueue the asynchronous read of this frame's counters into counters64 (a pinned 64-byte host
        buffer: a torch uint8 tensor or a numpy array); decode with frame_stats_decode once the stream passed."""
        ptr = counters64.data_ptr() if hasattr(counters64, "data_ptr") else counters64.ctypes.data
        _capi.check(_capi.lib().vh_frame_stats_enqueue(self.handle, C.c_void_p(ptr), _stream_handle(stream)),
                    self.handle)

    def frame_stats_decode(self, counters64):
        ptr = counters64.data_ptr() if hasattr(counters64, "data_ptr") else counters64.ctypes.data
        s = _capi.VhFrameStats()
        _capi.check(_capi.lib().vh_frame_stats_decode(self.handle, C.c_void_p(ptr), C.byref(s)), self.handle)
        return {f: getattr(s, f) for f, _ in s._fields_}

    def profile(self, enable=True):
        """Stage timing of vh_integrate with CUDA events (see read_profile)."""
        _capi.check(_capi.lib().vh_profile_enable(self.handle, 1 if enable else 0), self.handle)

    def read_profile(self):
        """({'filter', 'allocate', 'prepare', 'update', 'integrate': ms}, frames) accumulated since the last
        read; prepare = active-voxel list or normal map, update = layer update, integrate = their sum."""
        ms = (C.c_double * 4)()
        n = C.c_uint64()
        _capi.check(_capi.lib().vh_profile_read(self.handle, ms, C.byref(n)), self.handle)
        return {"filter": ms[0], "allocate": ms[1], "prepare": ms[2], "update": ms[3],
                "integrate": ms[2] + ms[3]}, n.value

    def block_keys(self):
        """gpuVolumeCacheBlockKeys: (N, 3) int32 in allocation order."""
        n = self.block_count()
        keys = np.zeros((n, 3), np.int32)
        if n:
            _capi.check(_capi.lib().vh_export_blocks(self.handle, 0, n, keys.ctypes.data_as(C.POINTER(C.c_int32)),
                                                     None, 0, None), self.handle)
        return keys

    def export_blocks(self, first=0, count=None):
        """(keys (N,3) int32, voxels (N,512,6,3,4) raw 32-bit words) in the reference Voxel layout
        (gpuVolumeCacheFlatBlocks); the last word of each layer is the packed normal (uint32)."""
        total = self.block_count()
        count = total - first if count is None else count
        keys = np.zeros((count, 3), np.int32)
        vox = np.zeros((count, 512, 6, 3, 4), np.uint32)
        if count:
            _capi.check(_capi.lib().vh_export_blocks(self.handle, first, count,
                                                     keys.ctypes.data_as(C.POINTER(C.c_int32)),
                                                     C.c_void_p(vox.ctypes.data), 0, None), self.handle)
        return keys, vox


    def import_blocks(self, keys, voxels):
        """applyFlatBlocks: insert/overwrite blocks from (keys (N,3) int32, voxels in the reference layout as
        returned by export_blocks); keys must be unique.  Checkpoint / resume."""
        k = np.ascontiguousarray(keys, np.int32).reshape(-1, 3)
        v = np.ascontiguousarray(voxels).view(np.uint32).reshape(k.shape[0], -1)
        _capi.check(_capi.lib().vh_import_blocks(self.handle, k.ctypes.data_as(C.POINTER(C.c_int32)),
                                                 C.c_void_p(v.ctypes.data), k.shape[0], 0, None), self.handle)


    def evict_blocks(self, min_age_frames, target_blocks=0, native=True):
        """Evicts the blocks not updated within the last min_age_frames frames (and, with target_blocks, the oldest
        further ones until exactly target_blocks remain); returns (keys (N,3) int32, data): the volume's own block
        images (N, block bytes) uint8 for restore_blocks when native, else the reference Voxel layout as
        export_blocks returns it.  Host memory."""
        return self._evict_into(min_age_frames, target_blocks, native, self.block_count())

    def _evict_into(self, min_age_frames, target_blocks, native, hint):
        bpb = (98304 if self.layer_format == 1 else 147456) if native else 147456
        cap = max(int(hint), 1)
        while True:
            keys = np.zeros((cap, 3), np.int32)
            data = np.zeros((cap, bpb), np.uint8)
            n = C.c_uint64()
            st = _capi.lib().vh_evict_blocks(self.handle, int(min_age_frames), int(target_blocks), 1 if native else 0,
                                             keys.ctypes.data_as(C.POINTER(C.c_int32)), C.c_void_p(data.ctypes.data),
                                             cap, 0, C.byref(n), None)
            if st == _capi.VH_ERR_BUFFER_TOO_SMALL:
                cap = int(n.value)
                continue
            _capi.check(st, self.handle)
            m = int(n.value)
            if native:
                return keys[:m], data[:m]
            return keys[:m], data[:m].view(np.uint32).reshape(m, 512, 6, 3, 4)

    def restore_blocks(self, keys, data):
        """Puts back blocks saved by evict_blocks(native=True), bit for bit."""
        k = np.ascontiguousarray(keys, np.int32).reshape(-1, 3)
        d = np.ascontiguousarray(data)
        _capi.check(_capi.lib().vh_restore_blocks(self.handle, k.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  C.c_void_p(d.ctypes.data), k.shape[0], 0, None), self.handle)


class TsdfIntegrationBackend:
    """reconstruction_backend.h:18-42, GPU only."""

    def __init__(self, preference=ComputeBackendPreference.AUTO):
        if isinstance(preference, str):
            preference = parse_compute_backend_preference(preference)
        if preference is ComputeBackendPreference.CPU:
            raise RuntimeError("the GB300 backend has no CPU path; use the reference CPU build for kCpu")
        ok, msg = query_cuda_backend_status()
        if not ok:
            raise RuntimeError("GPU backend requested but CUDA is unavailable: " + msg)
        self._description = "GPU (GB300 CUDA%s)" % (", auto-selected" if preference is ComputeBackendPreference.AUTO
                                                       else "")

    @property
    def description(self):
        return self._description

    @property
    def uses_gpu(self):
        return True

    def integrate(self, volume: VoxelHashTSDF, frame: DepthFrame, T_wc, allocation_stride=1, stream=None,
                  synchronize=True):
        integrate_depth_frame_cuda(volume, frame, T_wc, allocation_stride, stream=stream, synchronize=synchronize)

    def extract_mesh(self, volume: VoxelHashTSDF, iso_level=0.0, stream=None):
        return extract_mesh_cuda(volume, iso_level, stream=stream)

    def block_count(self, volume: VoxelHashTSDF):
        return volume.block_count()

    def observed_voxel_count(self, volume: VoxelHashTSDF):
        return volume.observed_voxel_count()


def integrate_depth_frame_cuda(volume: VoxelHashTSDF, frame: DepthFrame, T_wc, allocation_stride=1, stream=None,
                               synchronize=True):
    """Filter -> allocate -> integrate one frame.  With synchronize=False the call only enqueues work and
    device-side errors surface at the next volume.synchronize()."""
    ptr, on_dev, _keep = frame._pointer()
    K = _capi.intrinsics(frame.intrinsics)
    P = _capi.pose(T_wc)
    s = _stream_handle(stream)
    _capi.check(_capi.lib().vh_integrate(volume.handle, ptr, on_dev, C.byref(K), C.byref(P), int(allocation_stride),
                                         s), volume.handle)
    if synchronize:
        volume.synchronize(stream)


_transient = {}


def _next_pow2(x):
    return 1 if x <= 1 else 1 << (int(x) - 1).bit_length()


def allocate_active_blocks_cuda(frame: DepthFrame, T_wc, voxel_size, truncation_distance, allocation_stride=1,
                                volume: VoxelHashTSDF | None = None, stream=None):
    """Unique block keys (N, 3) int32 of one frame (unordered).

    Without ``volume`` the call is stateless like the reference: a keys-only table sized by the reference's
    rule, nextPow2(2 * max(2048, 16 * samples)) (cuda_block_allocator.cu:322-323), is cleared and reused.
    With ``volume`` the blocks are added to that volume.  Overflow raises VhError (the reference throws
    CudaActiveBlockAllocationFallback)."""
    K = frame.intrinsics
    stride = max(1, int(allocation_stride))
    samples = ((K.width + stride - 1) // stride) * ((K.height + stride - 1) // stride)
    if samples == 0:
        return np.zeros((0, 3), np.int32)
    if volume is None:
        cap = _next_pow2(2 * max(2048, 16 * samples))
        key = (float(voxel_size), float(truncation_distance), cap)
        volume = _transient.get(key)
        if volume is None:
            _transient.clear()
            volume = VoxelHashTSDF(voxel_size, truncation_distance, hash_buckets=cap, max_blocks=0)
            _transient[key] = volume
        else:
            volume.reset(stream)
    ptr, on_dev, _keep = frame._pointer()
    Kc = _capi.intrinsics(K)
    P = _capi.pose(T_wc)
    n = C.c_size_t()
    s = _stream_handle(stream)
    _capi.check(_capi.lib().vh_allocate(volume.handle, ptr, on_dev, C.byref(Kc), C.byref(P), stride, None, 0,
                                        C.byref(n), s), volume.handle)
    return visible_block_keys(volume, stream)


def visible_block_keys(volume: VoxelHashTSDF, stream=None):
    """(N, 3) int32 keys of the blocks the last integrated/allocated frame touched (unordered)."""
    n = C.c_size_t()
    s = _stream_handle(stream)
    _capi.check(_capi.lib().vh_visible_block_keys(volume.handle, None, 0, C.byref(n), s), volume.handle)
    keys = np.zeros((max(1, n.value), 3), np.int32)
    _capi.check(_capi.lib().vh_visible_block_keys(volume.handle, keys.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  keys.shape[0], C.byref(n), s), volume.handle)
    return keys[:n.value].copy()


class VolumeBatch:
    """Many volumes fused together (vh_batch_*): each integrate() is one step in which every active scene
    integrates one device-resident depth frame, as three work-queue kernels over all scenes: launched one by one
    (use_graph False), as one CUDA graph launch (True), or as one persistent cooperative launch
    (use_graph="persistent").  Volumes need algorithm.normal_mode 1 and the same fast_math setting."""

    def __init__(self, volumes, use_graph=True):
        self.volumes = list(volumes)
        handles = (C.c_void_p * len(self.volumes))(*[v.handle.value for v in self.volumes])
        h = C.c_void_p()
        mode = 2 if use_graph == "persistent" else (1 if use_graph else 0)
        _capi.check(_capi.lib().vh_batch_create(handles, len(self.volumes), mode, C.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            _capi.lib().vh_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def integrate(self, depths, intrinsics, poses, stride=1, stream=None):
        """depths[i]: contiguous float32 CUDA tensor of scene i's frame, or None to skip scene i this step."""
        n = len(self.volumes)
        ptrs = (C.c_void_p * n)()
        Ks = (_capi.VhIntrinsics * n)()
        Ps = (_capi.VhPose * n)()
        act = (C.c_int32 * n)()
        for i in range(n):
            if depths[i] is None:
                continue
            d = depths[i]
            if not (hasattr(d, "is_cuda") and d.is_cuda and d.is_contiguous()):
                raise ValueError("batch depth must be a contiguous CUDA tensor")
            if d.numel() != intrinsics[i].width * intrinsics[i].height:
                raise ValueError("depth size does not match the intrinsics of scene %d" % i)
            ptrs[i] = d.data_ptr()
            Ks[i] = _capi.intrinsics(intrinsics[i])
            Ps[i] = _capi.pose(poses[i])
            act[i] = 1
        self._keep = depths  # the kernels read the tensors asynchronously
        _capi.check(_capi.lib().vh_batch_integrate(self.handle, ptrs, Ks, Ps, act, int(stride), _stream_handle(stream)))


def raycast_depth(volume: VoxelHashTSDF, intrinsics, T_wc, min_depth=0.1, max_depth=8.0, step_voxels=0.5, stream=None,
                  device_out=None):
    """Depth map (H, W) float32 of the fused surface seen from T_wc (vh_raycast_depth); 0 = no hit.  With
    device_out (a torch device), a CUDA tensor is returned instead of a numpy array."""
    import torch
    K = _capi.intrinsics(intrinsics)
    out = torch.empty((intrinsics.height, intrinsics.width), dtype=torch.float32, device="cuda")
    s = _stream_handle(stream)
    _capi.check(_capi.lib().vh_raycast_depth(volume.handle, C.byref(K), C.byref(_capi.pose(T_wc)), float(min_depth),
                                             float(max_depth), float(step_voxels), C.c_void_p(out.data_ptr()), s),
                volume.handle)
    if device_out is not None:
        return out
    volume.synchronize(stream)
    return out.cpu().numpy()


def extract_mesh_cuda(volume: VoxelHashTSDF, iso_level=0.0, stream=None, device_out=None, recent_frames=0):
    """Triangle soup (N, 9) float32 (v0, v1, v2).  With device_out (a torch tensor factory device), the soup
    is returned as a CUDA tensor instead of a host array.  recent_frames > 0: incremental meshing, only the
    blocks updated within that many frames (vh_extract_mesh_recent)."""
    n = C.c_size_t()
    s = _stream_handle(stream)
    if recent_frames:
        _capi.check(_capi.lib().vh_extract_mesh_recent(volume.handle, float(iso_level), int(recent_frames),
                                                       C.byref(n), s), volume.handle)
    else:
        _capi.check(_capi.lib().vh_extract_mesh(volume.handle, float(iso_level), C.byref(n), s), volume.handle)
    if device_out is not None:
        import torch
        out = torch.empty((n.value, 9), dtype=torch.float32, device=device_out)
        if n.value:
            _capi.check(_capi.lib().vh_copy_mesh(volume.handle, C.c_void_p(out.data_ptr()), n.value, 1, s),
                        volume.handle)
        return out
    out = np.zeros((n.value, 9), np.float32)
    if n.value:
        _capi.check(_capi.lib().vh_copy_mesh(volume.handle, C.c_void_p(out.ctypes.data), n.value, 0, s),
                    volume.handle)
    return out


def extract_mesh_indexed(volume: VoxelHashTSDF, iso_level=0.0, stream=None, recent_frames=0):
    """Indexed mesh (vertices (V, 3) float32, faces (F, 3) int32) welded on the device (vh_weld_mesh): soup
    vertices merged when bit-identical, numbered by first use; collapsed and zero-area faces dropped."""
    n = C.c_size_t()
    s = _stream_handle(stream)
    if recent_frames:
        _capi.check(_capi.lib().vh_extract_mesh_recent(volume.handle, float(iso_level), int(recent_frames),
                                                       C.byref(n), s), volume.handle)
    else:
        _capi.check(_capi.lib().vh_extract_mesh(volume.handle, float(iso_level), C.byref(n), s), volume.handle)
    nv, nf = C.c_size_t(), C.c_size_t()
    _capi.check(_capi.lib().vh_weld_mesh(volume.handle, C.byref(nv), C.byref(nf), s), volume.handle)
    verts = np.zeros((nv.value, 3), np.float32)
    faces = np.zeros((nf.value, 3), np.int32)
    _capi.check(_capi.lib().vh_copy_welded_mesh(volume.handle, C.c_void_p(verts.ctypes.data), nv.value,
                                                C.c_void_p(faces.ctypes.data), nf.value, 0, s), volume.handle)
    return verts, faces


def gpu_volume_cache_block_count(volume: VoxelHashTSDF):
    return volume.block_count()


def gpu_volume_cache_observed_voxel_count(volume: VoxelHashTSDF):
    return volume.observed_voxel_count()


def gpu_volume_cache_block_keys(volume: VoxelHashTSDF):
    return volume.block_keys()
