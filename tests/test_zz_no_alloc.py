"""vh_allocate_static_scratch: the allocation entry point for callers that cannot allocate device memory
once running (real-time tracking loops that forbid allocator calls, applications whose own pool owns the
whole device).  It keeps its hash table in a fixed static device array instead of cudaMalloc'd scratch.

Checked through the C ABI against the existing entry point (vh_allocate on a keys-only volume, via
allocate_active_blocks_cuda) on two calls in a row: the block keys are integers, so the sets must be equal
exactly.  The second call must not see the first call's keys, which stay in the shared array.  This file is
named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _sorted(k):
    k = np.asarray(k, np.int32).reshape(-1, 3)
    return k[np.lexsort((k[:, 2], k[:, 1], k[:, 0]))]


def _static_allocate(capi, depth_dev, K, P, voxel_size, truncation, stride, max_keys):
    keys = torch.full((max_keys, 3), -7, dtype=torch.int32, device="cuda")
    n = C.c_size_t()
    Kc = capi.intrinsics(K)
    Pc = capi.pose(P)
    st = capi.lib().vh_allocate_static_scratch(C.c_void_p(depth_dev.data_ptr()), C.byref(Kc), C.byref(Pc),
                                               voxel_size, truncation, stride, C.c_void_p(keys.data_ptr()), max_keys,
                                               C.byref(n), None)
    return st, keys[: n.value].cpu().numpy()


def test_static_scratch_matches_vh_allocate_twice(product_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import _capi, backend, scenes
    sc = scenes.orbit_scene(seed=21, frames=16, width=96, height=72, fx=83.1, fy=83.1, cx=48.0, cy=36.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    K = sc.intrinsics
    for f, stride in ((0, 1), (9, 2)):  # two calls in a row with different frames, poses and strides
        d = scenes.render_depth(sc, f)
        st, got = _static_allocate(_capi, torch.from_numpy(d).cuda(), K, sc.poses[f], sc.voxel_size, sc.truncation,
                                   stride, 200000)
        assert st == _capi.VH_OK, _capi.VhError(st, "").args[0]
        want = backend.allocate_active_blocks_cuda(backend.DepthFrame(K, d), sc.poses[f], sc.voxel_size,
                                                   sc.truncation, stride)
        assert got.shape[0] > 0
        assert np.array_equal(_sorted(got), _sorted(want))


def test_static_scratch_rejects_frames_beyond_its_capacity(product_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import _capi, scenes
    K = scenes.Intrinsics(640, 480, 525.0, 525.0, 319.5, 239.5)  # 307,200 samples at stride 1 > 32,768
    d = torch.ones((480, 640), dtype=torch.float32, device="cuda")
    st, _ = _static_allocate(_capi, d, K, scenes.Pose(), 0.005, 0.02, 1, 16)
    assert st == _capi.VH_ERR_CAPACITY
    st, keys = _static_allocate(_capi, d, K, scenes.Pose(), 0.005, 0.02, 4, 200000)  # 160x120 samples fit
    assert st == _capi.VH_OK and keys.shape[0] > 0
