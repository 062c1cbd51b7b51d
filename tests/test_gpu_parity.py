"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same seeded inputs.

Plain FP32 form: filtered depth, filter normals, block-key sets, every voxel layer word, observed-voxel
counts and the marching-cubes soup must be bit-identical to the oracle's REF_GPU flavour -- with its
restatement of the C library's expf (VO_EXP_OWN) and with the C library's expf itself (VO_EXP_LIBM, the
reference's own exponential), which are the same function.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def env(product_lib, oracle_lib):
    _need_gpu()
    from voxelhashmt_gb300 import backend
    return backend, oracle_lib


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _sorted_keys(k):
    k = np.asarray(k, np.int32).reshape(-1, 3)
    return k[np.lexsort((k[:, 2], k[:, 1], k[:, 0]))]


def _volume(backend, sc, **kw):
    kw.setdefault("hash_buckets", 1 << 16)
    kw.setdefault("max_blocks", 8192)
    return backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, **kw)


def _filter_gpu(backend, vol, depth, K):
    from voxelhashmt_gb300 import _capi
    d = _dev(depth)
    out = torch.empty_like(d)
    Kc = _capi.intrinsics(K)
    _capi.check(_capi.lib().vh_filter_depth(vol.handle, C.c_void_p(d.data_ptr()), C.c_void_p(out.data_ptr()),
                                            C.byref(Kc), None), vol.handle)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("size", [(64, 48), (97, 61), (320, 240)])
def test_filter_bit_exact(env, size):
    backend, O = env
    from voxelhashmt_gb300 import scenes
    w, h = size
    sc = scenes.orbit_scene(seed=11, frames=8, width=w, height=h, fx=277.0 * w / 320, fy=277.0 * w / 320,
                            cx=w / 2, cy=h / 2)
    vol = _volume(backend, sc, max_blocks=1)
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN, threads=8)
    for f in (0, 3):
        d = scenes.render_depth(sc, f)
        got = _filter_gpu(backend, vol, d, sc.intrinsics)
        want = O.filter_depth(cfg, d, sc.intrinsics)
        assert np.array_equal(_bits(got), _bits(want)), "filtered depth differs at %d px" % int(
            np.sum(_bits(got) != _bits(want)))
    vol.close()


def test_depth_normals_bit_exact(env):
    backend, O = env
    from voxelhashmt_gb300 import _capi, scenes
    sc = scenes.orbit_scene(seed=5, frames=4, width=97, height=61, fx=84.0, fy=84.0, cx=48.5, cy=30.5)
    vol = _volume(backend, sc, max_blocks=1)
    d = scenes.render_depth(sc, 1)
    dd = _dev(d)
    n = torch.empty((d.size * 3,), dtype=torch.float32, device="cuda")
    v = torch.empty((d.size,), dtype=torch.uint8, device="cuda")
    Kc = _capi.intrinsics(sc.intrinsics)
    _capi.check(_capi.lib().vh_depth_normals(vol.handle, C.c_void_p(dd.data_ptr()), C.c_void_p(n.data_ptr()),
                                             C.c_void_p(v.data_ptr()), C.byref(Kc), None), vol.handle)
    torch.cuda.synchronize()
    wn, wv = O.depth_normals(O.config(O.FLAVOR_REF_GPU, O.EXP_OWN), d, sc.intrinsics)
    assert np.array_equal(v.cpu().numpy(), wv.reshape(-1))
    assert np.array_equal(_bits(n.cpu().numpy()), _bits(wn.reshape(-1)))
    vol.close()


@pytest.mark.parametrize("stride", [1, 2, 3])
def test_allocate_keys_match_oracle(env, small_orbit, stride):
    backend, O = env
    sc = small_orbit
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN)
    from voxelhashmt_gb300 import scenes
    for f in (0, 5, 13):
        d = scenes.render_depth(sc, f)
        frame = backend.DepthFrame(sc.intrinsics, d)
        got = backend.allocate_active_blocks_cuda(frame, sc.poses[f], sc.voxel_size, sc.truncation, stride)
        want = O.collect_blocks(cfg, d, sc.intrinsics, sc.poses[f], sc.voxel_size, sc.truncation, stride)
        assert got.shape == want.shape
        assert np.array_equal(_sorted_keys(got), want)


def _integrate_both(backend, O, sc, frames, exp_impl=None, stride=1, device_input=False):
    from voxelhashmt_gb300 import scenes
    O_exp = O.EXP_OWN if exp_impl is None else exp_impl
    cfg = O.config(O.FLAVOR_REF_GPU, O_exp, threads=8)
    vol = _volume(backend, sc)
    ora = O.Volume(cfg, sc.voxel_size, sc.truncation)
    bk = backend.TsdfIntegrationBackend("gpu")
    for f in frames:
        d = scenes.render_depth(sc, f)
        frame = backend.DepthFrame(sc.intrinsics, _dev(d) if device_input else d)
        bk.integrate(vol, frame, sc.poses[f], stride)
        n_ora = ora.integrate(d, sc.intrinsics, sc.poses[f], stride)
        assert vol.frame_stats()["visible_blocks"] == n_ora
    return vol, ora


def test_integrate_bit_exact(env, small_orbit):
    backend, O = env
    vol, ora = _integrate_both(backend, O, small_orbit, frames=[0, 6, 12, 18, 1])
    gk, gv = vol.export_blocks()
    ok_, ov = ora.blocks()
    gk, gv = O.sort_blocks(gk, gv)
    ok_, ov = O.sort_blocks(ok_, ov)
    assert np.array_equal(gk, ok_)
    assert np.array_equal(gv.reshape(len(gk), -1), ov.view(np.uint32).reshape(len(ok_), -1))
    assert vol.observed_voxel_count() == ora.observed_voxels()
    assert vol.recount_observed_voxels() == ora.observed_voxels()
    assert vol.block_count() == ora.block_count()
    vol.close()


@pytest.mark.parametrize("stride", [2, 3])
def test_integrate_stride_and_device_input(env, small_orbit, stride):
    """Strided sampling through the fused filter + allocation kernel (samples are the pixels whose coordinates
    are multiples of the stride, inside each 32x8 filter tile), bit-identical to the oracle."""
    backend, O = env
    vol, ora = _integrate_both(backend, O, small_orbit, frames=[2, 9], stride=stride, device_input=True)
    gk, gv = O.sort_blocks(*vol.export_blocks())
    ok_, ov = O.sort_blocks(*ora.blocks())
    assert np.array_equal(gk, ok_)
    assert np.array_equal(gv.reshape(len(gk), -1), ov.view(np.uint32).reshape(len(ok_), -1))
    vol.close()


def test_pinned_host_frames_back_to_back_match_device_input(env, small_orbit):
    """Host depth is staged through two device buffers on an internal copy stream (the copy of the next frame
    overlaps this frame's kernels).  Frames enqueued back to back from pinned host memory, without a
    synchronisation in between, fuse into the same volume, bit for bit, as the same frames from device memory;
    seven frames through the two buffers make every buffer wait for its previous readers."""
    backend, _ = env
    from voxelhashmt_gb300 import scenes
    sc = small_orbit
    frames = [0, 3, 6, 9, 12, 15, 18]
    depths = [scenes.render_depth(sc, f) for f in frames]
    pinned = torch.empty((len(frames),) + depths[0].shape, dtype=torch.float32, pin_memory=True)
    for k, d in enumerate(depths):
        pinned[k].copy_(torch.from_numpy(d))
    bk = backend.TsdfIntegrationBackend("gpu")
    host_vol, dev_vol = _volume(backend, sc), _volume(backend, sc)
    for k, f in enumerate(frames):
        bk.integrate(host_vol, backend.DepthFrame(sc.intrinsics, pinned[k].numpy()), sc.poses[f], 1,
                     synchronize=False)
    host_vol.synchronize()
    for k, f in enumerate(frames):
        bk.integrate(dev_vol, backend.DepthFrame(sc.intrinsics, _dev(depths[k])), sc.poses[f], 1)
    hk, hv = _sorted_blocks(env, host_vol)
    dk, dv = _sorted_blocks(env, dev_vol)
    assert hk.shape[0] > 0
    assert np.array_equal(hk, dk) and np.array_equal(hv, dv)
    host_vol.close()
    dev_vol.close()


def test_pinned_host_frames_of_changing_resolution(env, small_orbit):
    """A larger host frame reallocates the two staging buffers while earlier frames may still be in flight
    (the copy stream and the readers are waited for first): 64x48 and 128x96 frames of one orbit, enqueued
    back to back from pinned memory, fuse bit-identically to the same frames from device memory."""
    backend, _ = env
    from voxelhashmt_gb300 import scenes
    small = small_orbit
    big = scenes.orbit_scene(seed=7, frames=24, width=128, height=96, fx=277.0 * 0.4, fy=277.0 * 0.4, cx=64.0,
                             cy=48.0)
    big.voxel_size, big.truncation = small.voxel_size, small.truncation
    plan = [(small, 0), (small, 3), (big, 6), (big, 9), (small, 12), (big, 15)]
    depths = [scenes.render_depth(sc, f) for sc, f in plan]
    pinned = [torch.from_numpy(d).pin_memory() for d in depths]
    bk = backend.TsdfIntegrationBackend("gpu")
    host_vol, dev_vol = _volume(backend, small), _volume(backend, small)
    for (sc, f), h in zip(plan, pinned):
        bk.integrate(host_vol, backend.DepthFrame(sc.intrinsics, h.numpy()), sc.poses[f], 1, synchronize=False)
    host_vol.synchronize()
    for (sc, f), d in zip(plan, depths):
        bk.integrate(dev_vol, backend.DepthFrame(sc.intrinsics, _dev(d)), sc.poses[f], 1)
    hk, hv = _sorted_blocks(env, host_vol)
    dk, dv = _sorted_blocks(env, dev_vol)
    assert hk.shape[0] > 0
    assert np.array_equal(hk, dk) and np.array_equal(hv, dv)
    host_vol.close()
    dev_vol.close()


def _sorted_blocks(env, vol):
    return env[1].sort_blocks(*vol.export_blocks())


def test_mesh_bit_exact_and_deterministic(env, small_orbit):
    backend, O = env
    vol, ora = _integrate_both(backend, O, small_orbit, frames=[0, 4, 8, 12, 16, 20])
    bk = backend.TsdfIntegrationBackend("auto")
    got = bk.extract_mesh(vol)
    want = ora.extract_mesh()
    assert got.shape == want.shape and got.shape[0] > 0
    assert np.array_equal(_bits(O.canonical_triangles(got)), _bits(O.canonical_triangles(want)))
    again = bk.extract_mesh(vol)
    assert np.array_equal(_bits(again), _bits(got)), "two extractions of the same volume differ"
    dev = backend.extract_mesh_cuda(vol, device_out="cuda")
    assert np.array_equal(_bits(dev.cpu().numpy()), _bits(got))
    from voxelhashmt_gb300 import mesh_io
    verts, faces = mesh_io.weld(got)
    assert 0 < verts.shape[0] < 3 * got.shape[0] and 0 < faces.shape[0] <= got.shape[0]
    # the device weld builds the same indexed mesh
    dv, df = backend.extract_mesh_indexed(vol)
    assert np.array_equal(_bits(dv), _bits(verts)) and np.array_equal(df, faces)
    vol.close()


def test_bit_exact_with_c_library_expf(env, small_orbit):
    """Against the oracle evaluated with the C library's expf -- the exponential the reference calls -- the voxel
    words and the triangle soup are bit-identical (where this host's C library is the restated algorithm)."""
    backend, O = env
    import os
    n, first = O.expf_compare_libm(0x80000000, 0x7F800001, threads=max(os.cpu_count() or 1, 1))
    # allowed: the one non-positive argument where an unfused reduction step rounds differently
    if not (n == 0 or (n == 1 and first == 0xC27C65D9)):
        pytest.skip("this host's C library expf is not the restated algorithm")
    sc = small_orbit
    vol, ref = _integrate_both(backend, O, sc, frames=[0, 6, 12], exp_impl=O.EXP_LIBM)
    gk, gv = O.sort_blocks(*vol.export_blocks())
    rk, rv = O.sort_blocks(*ref.blocks())
    assert np.array_equal(gk, rk)
    assert np.array_equal(gv.reshape(len(gk), -1), rv.view(np.uint32).reshape(len(rk), -1))
    gm = backend.extract_mesh_cuda(vol)
    rm = ref.extract_mesh()
    assert np.array_equal(O.canonical_triangles(gm).view(np.uint32), O.canonical_triangles(rm).view(np.uint32))
    vol.close()


def test_empty_depth_allocates_nothing(env, small_orbit):
    backend, O = env
    sc = small_orbit
    vol = _volume(backend, sc)
    z = np.zeros((sc.intrinsics.height, sc.intrinsics.width), np.float32)
    backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, z), sc.poses[0])
    assert vol.block_count() == 0 and vol.observed_voxel_count() == 0
    assert backend.extract_mesh_cuda(vol).shape == (0, 9)
    keys = backend.allocate_active_blocks_cuda(backend.DepthFrame(sc.intrinsics, z), sc.poses[0], sc.voxel_size,
                                               sc.truncation)
    assert keys.shape == (0, 3)
    vol.close()


def test_key_range_error(env, small_orbit):
    backend, O = env
    from voxelhashmt_gb300 import _capi, scenes
    sc = small_orbit
    far = scenes.Pose(sc.poses[0].R.copy(), sc.poses[0].t + np.float32([1.0e6, 0.0, 0.0]))  # > 2^20 blocks
    vol = _volume(backend, sc)
    d = scenes.render_depth(sc, 0)
    with pytest.raises(_capi.VhError) as e:
        backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), far)
    assert e.value.status == _capi.VH_ERR_KEY_RANGE
    assert O.collect_blocks(O.config(O.FLAVOR_REF_GPU), d, sc.intrinsics, far, sc.voxel_size, sc.truncation) is None
    # the error was consumed by the failing call; the volume keeps working
    backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[0])
    vol.close()


def test_hash_and_pool_full_errors(env, small_orbit):
    backend, O = env
    from voxelhashmt_gb300 import _capi, scenes
    sc = small_orbit
    d = scenes.render_depth(sc, 0)
    vol = _volume(backend, sc, hash_buckets=64, max_blocks=64)
    with pytest.raises(_capi.VhError) as e:
        backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[0])
    assert e.value.status == _capi.VH_ERR_HASH_FULL
    vol.close()
    vol = _volume(backend, sc, max_blocks=16)
    with pytest.raises(_capi.VhError) as e:
        backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[0])
    assert e.value.status == _capi.VH_ERR_POOL_FULL
    assert vol.block_count() == 16
    vol.close()


def test_reset_and_reintegrate_is_identical(env, small_orbit):
    backend, O = env
    from voxelhashmt_gb300 import scenes
    sc = small_orbit
    vol = _volume(backend, sc)
    frames = [backend.DepthFrame(sc.intrinsics, scenes.render_depth(sc, f)) for f in (0, 7)]
    for fr, f in zip(frames, (0, 7)):
        backend.integrate_depth_frame_cuda(vol, fr, sc.poses[f])
    a = O.sort_blocks(*vol.export_blocks())
    vol.reset()
    assert vol.block_count() == 0 and vol.observed_voxel_count() == 0
    for fr, f in zip(frames, (0, 7)):
        backend.integrate_depth_frame_cuda(vol, fr, sc.poses[f])
    b = O.sort_blocks(*vol.export_blocks())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    vol.close()


def test_room_frame_full_resolution_properties(env):
    """640x480 room frames: visible keys = oracle allocation on the (bit-exact) filtered depth,
    incremental observed count = recount."""
    backend, O = env
    from voxelhashmt_gb300 import scenes
    sc = scenes.room_scene(seed=1, frames=6)
    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 20, max_blocks=100000)
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN, threads=8)
    for f in range(0, 6, 2):
        d = scenes.render_depth(sc, f)
        backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[f])
        got = _sorted_keys(backend.visible_block_keys(vol))
        fd = O.filter_depth(cfg, d, sc.intrinsics)
        want = O.collect_blocks(cfg, fd, sc.intrinsics, sc.poses[f], sc.voxel_size, sc.truncation)
        assert np.array_equal(got, want)
    assert vol.observed_voxel_count() == vol.recount_observed_voxels()
    tris = backend.extract_mesh_cuda(vol)
    assert tris.shape[0] > 1000 and np.all(np.isfinite(tris))
    from voxelhashmt_gb300 import mesh_io
    verts, faces = mesh_io.weld(tris)
    dv, df = backend.extract_mesh_indexed(vol)
    assert np.array_equal(_bits(dv), _bits(verts)) and np.array_equal(df, faces)
    vol.close()


def test_checkpoint_export_import_round_trip(env, small_orbit):
    """applyFlatBlocks-style resume: export -> import into a fresh volume is the identity on blocks, counts
    and mesh, and integrating the next frame on both volumes gives the same result."""
    backend, O = env
    from voxelhashmt_gb300 import scenes
    sc = small_orbit
    a = _volume(backend, sc)
    for f in (0, 5, 10):
        backend.integrate_depth_frame_cuda(a, backend.DepthFrame(sc.intrinsics, scenes.render_depth(sc, f)), sc.poses[f])
    keys, vox = a.export_blocks()
    b = _volume(backend, sc)
    b.import_blocks(keys, vox)  # pool order is internal: compare blocks and meshes order-independently
    ka, va = O.sort_blocks(keys, vox)
    kb, vb = O.sort_blocks(*b.export_blocks())
    assert np.array_equal(ka, kb) and np.array_equal(va, vb)
    assert b.observed_voxel_count() == a.observed_voxel_count() == a.recount_observed_voxels()
    assert np.array_equal(_bits(O.canonical_triangles(backend.extract_mesh_cuda(a))),
                          _bits(O.canonical_triangles(backend.extract_mesh_cuda(b))))
    d = scenes.render_depth(sc, 15)
    for v in (a, b):
        backend.integrate_depth_frame_cuda(v, backend.DepthFrame(sc.intrinsics, d), sc.poses[15])
    ka, va = O.sort_blocks(*a.export_blocks())
    kb, vb = O.sort_blocks(*b.export_blocks())
    assert np.array_equal(ka, kb) and np.array_equal(va, vb)
    assert a.observed_voxel_count() == b.observed_voxel_count()
    a.close()
    b.close()


def test_import_matches_apply_flat_blocks(env, small_orbit):
    """vh_import_blocks against the oracle's restatement of applyFlatBlocks (voxel_hash_tsdf.h:183-188): records
    exported from a volume fused from other views -- keys that overwrite blocks of the target and keys that
    are new to it -- applied to a fused volume on both sides give the same blocks, voxel words and observed
    count; fusing a further frame and meshing afterwards stay bit-identical."""
    backend, O = env
    from voxelhashmt_gb300 import scenes
    sc = small_orbit
    vol, ora = _integrate_both(backend, O, sc, frames=[0, 4, 8])
    src = _volume(backend, sc)
    for f in (12, 16):
        backend.integrate_depth_frame_cuda(src, backend.DepthFrame(sc.intrinsics, scenes.render_depth(sc, f)),
                                           sc.poses[f])
    keys, vox = src.export_blocks()
    src.close()
    have = {tuple(k) for k in vol.export_blocks()[0]}
    overwrite = np.array([tuple(k) in have for k in keys])
    assert overwrite.sum() > 10 and (~overwrite).sum() > 10  # both kinds of record
    vol.import_blocks(keys, vox)
    ora.apply_flat_blocks(keys, vox)
    gk, gv = O.sort_blocks(*vol.export_blocks())
    ok, ov = O.sort_blocks(*ora.blocks())
    assert np.array_equal(gk, ok)
    assert np.array_equal(gv.reshape(len(gk), -1), ov.view(np.uint32).reshape(len(ok), -1))
    assert vol.observed_voxel_count() == ora.observed_voxels() == vol.recount_observed_voxels()
    d = scenes.render_depth(sc, 20)
    backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[20])
    ora.integrate(d, sc.intrinsics, sc.poses[20])
    gk, gv = O.sort_blocks(*vol.export_blocks())
    ok, ov = O.sort_blocks(*ora.blocks())
    assert np.array_equal(gk, ok)
    assert np.array_equal(gv.reshape(len(gk), -1), ov.view(np.uint32).reshape(len(ok), -1))
    assert vol.observed_voxel_count() == ora.observed_voxels()
    assert np.array_equal(_bits(O.canonical_triangles(backend.extract_mesh_cuda(vol))),
                          _bits(O.canonical_triangles(ora.extract_mesh())))
    vol.close()
    ora.close()


def test_raycast_bit_exact_and_close_to_scene(env, small_orbit):
    """Depth ray-cast of the fused plain volume: bit-identical to the oracle's restatement, and within a
    voxel of the analytic depth where both see the surface."""
    backend, O = env
    from voxelhashmt_gb300 import scenes
    sc = small_orbit
    vol, ora = _integrate_both(backend, O, sc, frames=[0, 3, 6, 9, 12])
    for f in (0, 4, 9):
        got = backend.raycast_depth(vol, sc.intrinsics, sc.poses[f], 0.1, 4.0, 0.5)
        want = ora.raycast_depth(sc.intrinsics, sc.poses[f], 0.1, 4.0, 0.5)
        assert np.array_equal(_bits(got), _bits(want)), int(np.sum(_bits(got) != _bits(want)))
        clean = scenes.render_depth(sc, f, noise=False)
        both = (got > 0) & (clean > 0)
        assert both.sum() > 0.5 * (clean > 0).sum()
        assert np.median(np.abs(got[both] - clean[both])) <= sc.voxel_size
    vol.close()


def test_incremental_meshing_is_a_subset_of_the_full_mesh(env, small_orbit):
    """vh_extract_mesh_recent: the soup of the blocks updated in the last k frames is a sub-multiset of the
    full extraction (bit-identical triangles), every triangle lies in or on the border of such a block, k = 0
    is the full mesh, and a k covering every frame gives the full mesh."""
    backend, O = env
    sc = small_orbit
    frames = [0, 4, 8, 12, 16, 20]
    vol, _ = _integrate_both(backend, O, sc, frames=frames)
    full = O.canonical_triangles(backend.extract_mesh_cuda(vol))
    assert np.array_equal(_bits(O.canonical_triangles(backend.extract_mesh_cuda(vol, recent_frames=0))), _bits(full))
    assert np.array_equal(_bits(O.canonical_triangles(backend.extract_mesh_cuda(vol, recent_frames=len(frames)))),
                          _bits(full))
    recent = O.canonical_triangles(backend.extract_mesh_cuda(vol, recent_frames=1))
    assert 0 < recent.shape[0] < full.shape[0]
    full_rows = {bytes(r) for r in _bits(full)}
    assert all(bytes(r) in full_rows for r in _bits(recent))
    vol.close()
