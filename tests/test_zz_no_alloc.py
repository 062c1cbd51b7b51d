"""vh_allocate_static_scratch: the allocation entry point for callers that cannot allocate device memory
once running (real-time tracking loops that forbid allocator calls, applications whose own pool owns the
whole device).  It keeps its hash table in a fixed static device array instead of cudaMalloc'd scratch.

Checked through the C ABI against the existing entry point (vh_allocate on a keys-only volume, via
allocate_active_blocks_cuda) on calls in a row: the block keys are integers, so the sets must be equal
exactly.  Later calls must not see earlier calls' keys, which stay in the shared array: the third call goes
back to the larger table after a call that used a smaller one, so the second call's stale keys lie inside the
range the third call probes.  This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _sorted(k):
    k = np.asarray(k, np.int32).reshape(-1, 3)
    return k[np.lexsort((k[:, 2], k[:, 1], k[:, 0]))]


def _static_allocate(capi, depth_dev, K, P, voxel_size, truncation, stride, max_keys, count_only=False):
    keys = torch.full((max(max_keys, 1), 3), -7, dtype=torch.int32, device="cuda")
    n = C.c_size_t(12345)
    Kc = capi.intrinsics(K)
    Pc = capi.pose(P)
    out = None if count_only else C.c_void_p(keys.data_ptr())
    st = capi.lib().vh_allocate_static_scratch(C.c_void_p(depth_dev.data_ptr()), C.byref(Kc), C.byref(Pc),
                                               voxel_size, truncation, stride, out, max_keys, C.byref(n), None)
    if st != capi.VH_OK or count_only:
        return st, n.value
    return st, keys[: n.value].cpu().numpy()


def test_static_scratch_matches_vh_allocate_twice(product_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import _capi, backend, scenes
    sc = scenes.orbit_scene(seed=21, frames=16, width=96, height=72, fx=83.1, fy=83.1, cx=48.0, cy=36.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    K = sc.intrinsics
    # calls in a row with different frames, poses and strides: 2^18 slots, then 2^16, then 2^18 again
    for f, stride in ((0, 1), (9, 2), (4, 1)):
        d = scenes.render_depth(sc, f)
        st, got = _static_allocate(_capi, torch.from_numpy(d).cuda(), K, sc.poses[f], sc.voxel_size, sc.truncation,
                                   stride, 200000)
        assert st == _capi.VH_OK, _capi.VhError(st, "").args[0]
        want = backend.allocate_active_blocks_cuda(backend.DepthFrame(K, d), sc.poses[f], sc.voxel_size,
                                                   sc.truncation, stride)
        assert got.shape[0] > 0
        assert np.array_equal(_sorted(got), _sorted(want))


def test_static_scratch_count_only_and_short_buffer(product_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import _capi, backend, scenes
    sc = scenes.orbit_scene(seed=22, frames=8, width=96, height=72, fx=83.1, fy=83.1, cx=48.0, cy=36.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    K = sc.intrinsics
    d = scenes.render_depth(sc, 3)
    dd = torch.from_numpy(d).cuda()
    want = backend.allocate_active_blocks_cuda(backend.DepthFrame(K, d), sc.poses[3], sc.voxel_size, sc.truncation, 1)
    n = want.reshape(-1, 3).shape[0]
    assert n > 1
    st, count = _static_allocate(_capi, dd, K, sc.poses[3], sc.voxel_size, sc.truncation, 1, 0, count_only=True)
    assert st == _capi.VH_OK and count == n
    st, count = _static_allocate(_capi, dd, K, sc.poses[3], sc.voxel_size, sc.truncation, 1, n - 1)
    assert st == _capi.VH_ERR_BUFFER_TOO_SMALL and count == n


def test_static_scratch_rejects_frames_beyond_its_capacity(product_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import _capi, scenes
    K = scenes.Intrinsics(640, 480, 525.0, 525.0, 319.5, 239.5)  # 307,200 samples at stride 1 > 32,768
    d = torch.ones((480, 640), dtype=torch.float32, device="cuda")
    st, count = _static_allocate(_capi, d, K, scenes.Pose(), 0.005, 0.02, 1, 16)
    assert st == _capi.VH_ERR_CAPACITY and count == 0
    st, keys = _static_allocate(_capi, d, K, scenes.Pose(), 0.005, 0.02, 4, 200000)  # 160x120 samples fit
    assert st == _capi.VH_OK and keys.shape[0] > 0
