"""Block eviction and restore (vh_evict_blocks / vh_restore_blocks), the pieces of the large streaming
configuration that keep a bounded pool over a long trajectory.

* Evicting the blocks not updated in the last frames splits the volume exactly: the survivors keep their voxel
  words, the evicted blocks come out with theirs (reference layout, or the pool's own image), and restoring the
  images gives back the volume that was never evicted -- keys, every voxel word, observed count and mesh -- for
  FP32 and FP16 storage.
* Fusing on after an eviction equals the oracle's volume with the same blocks removed, bit for bit.
* A target block count evicts the oldest blocks first, exactly down to the count; a short output buffer evicts
  nothing.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(product_lib, oracle_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import backend
    return backend, oracle_lib


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _volume(backend, sc, fp16):
    from voxelhashmt_gb300 import _capi
    algo = _capi.default_algorithm(allocation_mode=1, normal_mode=1, autotune=0) if fp16 else None
    return backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 16, max_blocks=16384,
                                 algorithm=algo, layer_format=1 if fp16 else 0)


def _fuse(backend, vol, sc, frames):
    from voxelhashmt_gb300 import scenes
    bk = backend.TsdfIntegrationBackend("gpu")
    for f in frames:
        bk.integrate(vol, backend.DepthFrame(sc.intrinsics, scenes.render_depth(sc, f)), sc.poses[f], 1)


def _rows(keys):
    return {tuple(int(x) for x in k) for k in np.asarray(keys).reshape(-1, 3)}


@pytest.mark.parametrize("fp16", [False, True])
def test_evict_splits_the_volume_and_restore_gives_it_back(env, small_orbit, fp16):
    backend, O = env
    sc = small_orbit
    frames = list(range(0, 24, 2))
    vol = _volume(backend, sc, fp16)
    _fuse(backend, vol, sc, frames)
    k0, v0 = O.sort_blocks(*vol.export_blocks())
    obs0 = vol.observed_voxel_count()
    m0 = O.canonical_triangles(backend.extract_mesh_cuda(vol))
    n0 = vol.block_count()
    # the reference-layout copy-out of a twin volume gives the evicted blocks' records
    twin = _volume(backend, sc, fp16)
    _fuse(backend, twin, sc, frames)
    tk, tv = twin.evict_blocks(4, native=False)
    twin.close()
    ek, ed = vol.evict_blocks(4, native=True)
    assert 0 < ek.shape[0] < n0 and vol.block_count() == n0 - ek.shape[0]
    assert _rows(tk) == _rows(ek)
    rk, rv = O.sort_blocks(*vol.export_blocks())
    assert _rows(rk).isdisjoint(_rows(ek)) and _rows(rk) | _rows(ek) == _rows(k0)
    index0 = {tuple(k): i for i, k in enumerate(k0.tolist())}
    sel = np.array([index0[tuple(k)] for k in rk.tolist()])
    assert np.array_equal(rv, v0[sel])  # survivors keep every word
    tks, tvs = O.sort_blocks(tk, tv)
    sel = np.array([index0[tuple(k)] for k in tks.tolist()])
    assert np.array_equal(tvs, v0[sel])  # evicted records as they were
    assert vol.observed_voxel_count() == vol.recount_observed_voxels() < obs0
    vol.restore_blocks(ek, ed)
    k1, v1 = O.sort_blocks(*vol.export_blocks())
    assert np.array_equal(k1, k0) and np.array_equal(v1, v0)
    assert vol.observed_voxel_count() == obs0 and vol.block_count() == n0
    assert np.array_equal(_bits(O.canonical_triangles(backend.extract_mesh_cuda(vol))), _bits(m0))
    vol.close()


def test_fusing_after_eviction_matches_the_oracle(env, small_orbit):
    backend, O = env
    from voxelhashmt_gb300 import scenes
    sc = small_orbit
    frames = list(range(0, 20, 2))
    vol = _volume(backend, sc, False)
    ora = O.Volume(O.config(O.FLAVOR_REF_GPU, O.EXP_OWN, threads=8), sc.voxel_size, sc.truncation)
    bk = backend.TsdfIntegrationBackend("gpu")
    for f in frames:
        d = scenes.render_depth(sc, f)
        bk.integrate(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[f], 1)
        ora.integrate(d, sc.intrinsics, sc.poses[f])
    ek, _ = vol.evict_blocks(3, native=True)
    assert ek.shape[0] > 0
    ora.remove_blocks(ek)
    for f in (20, 22, 1):  # frames that see evicted regions again re-allocate them empty
        d = scenes.render_depth(sc, f)
        bk.integrate(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[f], 1)
        n = ora.integrate(d, sc.intrinsics, sc.poses[f])
        assert vol.frame_stats()["visible_blocks"] == n
    gk, gv = O.sort_blocks(*vol.export_blocks())
    ok, ov = O.sort_blocks(*ora.blocks())
    assert np.array_equal(gk, ok)
    assert np.array_equal(gv.reshape(len(gk), -1), ov.view(np.uint32).reshape(len(ok), -1))
    assert vol.observed_voxel_count() == ora.observed_voxels()
    assert np.array_equal(_bits(O.canonical_triangles(backend.extract_mesh_cuda(vol))),
                          _bits(O.canonical_triangles(ora.extract_mesh())))
    vol.close()
    ora.close()


def test_target_evicts_oldest_first_and_short_buffers_evict_nothing(env, small_orbit):
    import ctypes as C
    backend, O = env
    from voxelhashmt_gb300 import _capi
    sc = small_orbit
    vol = _volume(backend, sc, False)
    _fuse(backend, vol, sc, list(range(0, 24, 2)))
    n0 = vol.block_count()
    keys = np.zeros((4, 3), np.int32)
    n = C.c_uint64()
    st = _capi.lib().vh_evict_blocks(vol.handle, 0, 0, 1, keys.ctypes.data_as(C.POINTER(C.c_int32)), None, 4, 0,
                                     C.byref(n), None)
    assert st == _capi.VH_ERR_BUFFER_TOO_SMALL and n.value == n0 and vol.block_count() == n0
    # the last frame's blocks are the youngest: keeping as many blocks as it touched keeps exactly those
    last = _rows(backend.visible_block_keys(vol))
    target = len(last)
    ek, _ = vol.evict_blocks(1 << 30, target_blocks=target, native=True)
    assert vol.block_count() == target and len(ek) == n0 - target
    assert _rows(vol.export_blocks()[0]) == last
    vol.close()


def test_target_evicts_exactly_down_to_the_count(env, small_orbit):
    """A target inside an age bin: the blocks of that age go in pool order until exactly target_blocks remain,
    and every younger block stays."""
    backend, O = env
    sc = small_orbit
    vol = _volume(backend, sc, False)
    _fuse(backend, vol, sc, list(range(0, 24, 2)))
    n0 = vol.block_count()
    last = _rows(backend.visible_block_keys(vol))
    target = len(last) + 3
    assert target < n0
    ek, _ = vol.evict_blocks(1 << 30, target_blocks=target, native=True)
    kept = _rows(vol.export_blocks()[0])
    assert vol.block_count() == target and len(ek) == n0 - target and len(kept) == target
    assert last <= kept
    vol.close()


@pytest.mark.parametrize("fp16", [False, True])
def test_evict_into_device_memory_matches_host(env, small_orbit, fp16):
    """Evicting into device buffers (the copy kernel stores into them directly) gives the same keys and block
    images as evicting into host memory, in both formats and both storage precisions."""
    import ctypes as C
    backend, O = env
    from voxelhashmt_gb300 import _capi
    sc = small_orbit
    frames = list(range(0, 20, 2))
    for native in (True, False):
        a, b = _volume(backend, sc, fp16), _volume(backend, sc, fp16)
        _fuse(backend, a, sc, frames)
        _fuse(backend, b, sc, frames)
        hk, hd = a.evict_blocks(6, native=native)
        n = len(hk)
        assert n > 0
        bpb = hd.reshape(n, -1).view(np.uint8).shape[1]
        dk = torch.zeros((n, 3), dtype=torch.int32, device="cuda")
        dd = torch.zeros((n, bpb), dtype=torch.uint8, device="cuda")
        cnt = C.c_uint64()
        _capi.check(_capi.lib().vh_evict_blocks(b.handle, 6, 0, 1 if native else 0,
                                                C.cast(C.c_void_p(dk.data_ptr()), C.POINTER(C.c_int32)),
                                                C.c_void_p(dd.data_ptr()), n, 1, C.byref(cnt), None), b.handle)
        assert cnt.value == n and b.block_count() == a.block_count()
        got = {tuple(k): bytes(d) for k, d in zip(dk.cpu().numpy().tolist(), dd.cpu().numpy())}
        want = {tuple(k): bytes(d) for k, d in zip(hk.tolist(), hd.reshape(n, -1).view(np.uint8))}
        assert got == want
        a.close()
        b.close()
