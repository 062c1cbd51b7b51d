"""Bit parity of the plain FP32 form at the benchmark configurations' own sizes.

* Small plain-method configuration: the orbit scene (ground plane, sphere r 0.5 m, 0.4 x 0.3 x 0.6 m box,
  centres seeded in a 1 m cube), 320x240, fx = fy = 277, cx 160, cy 120, camera orbit of radius 1.5 m at 0.8 m
  height, noise sigma 0.0012 z^2 plus 1 % dropouts; voxel 1 cm, truncation 4 cm, 2^16 hash buckets; every
  4th of its 64 frames (16 frames).
* Room configuration, first frames: 640x480, fx = fy = 525, the 4 x 5 x 3 m room with 40 seeded primitives,
  voxel 5 mm, truncation 2 cm, 2^20 buckets; frames 0-3 of the random walk.

Against the oracle with the C library's expf -- the reference's own arithmetic -- the GPU path is bit-identical:
each frame's visible block keys (allocation on the filtered depth), every voxel word of every block, the
observed-voxel count, and the marching-cubes triangle multiset.  The oracle runs with this host's C library
expf where it equals the restatement on the non-positive floats, or differs from it only at the one argument
where an unfused reduction step rounds differently (-0x1.f8cbb2p+5, a weight of 3.6e-28: a scene that met it
would fail the comparison); elsewhere the restatement (VO_EXP_OWN) stands in.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(product_lib, oracle_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import backend
    O = oracle_lib
    n, first = O.expf_compare_libm(0x80000000, 0x7F800001, threads=max(os.cpu_count() or 1, 1))
    libm_ok = n == 0 or (n == 1 and first == 0xC27C65D9)
    return backend, O, (O.EXP_LIBM if libm_ok else O.EXP_OWN)


def _sorted_keys(k):
    k = np.asarray(k, np.int32).reshape(-1, 3)
    return k[np.lexsort((k[:, 2], k[:, 1], k[:, 0]))]


def _fuse_and_compare(backend, O, exp_impl, sc, frames, hash_buckets, max_blocks):
    from voxelhashmt_gb300 import scenes
    threads = max(os.cpu_count() or 1, 1)
    cfg = O.config(O.FLAVOR_REF_GPU, exp_impl, threads=threads)
    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=hash_buckets, max_blocks=max_blocks)
    ora = O.Volume(cfg, sc.voxel_size, sc.truncation)
    bk = backend.TsdfIntegrationBackend("gpu")
    for f in frames:
        d = scenes.render_depth(sc, f)
        bk.integrate(vol, backend.DepthFrame(sc.intrinsics, torch.from_numpy(d).cuda()), sc.poses[f], 1)
        ora.integrate(d, sc.intrinsics, sc.poses[f])
        got = _sorted_keys(backend.visible_block_keys(vol))
        fd = O.filter_depth(cfg, d, sc.intrinsics)
        want = O.collect_blocks(cfg, fd, sc.intrinsics, sc.poses[f], sc.voxel_size, sc.truncation)
        assert np.array_equal(got, want), "frame %d: visible block keys differ" % f
    keys, vox = O.sort_blocks(*vol.export_blocks())
    okeys, ovox = O.sort_blocks(*ora.blocks())
    assert np.array_equal(keys, okeys)
    assert np.array_equal(vox.reshape(len(keys), -1), ovox.view(np.uint32).reshape(len(okeys), -1)), \
        "voxel words differ"
    assert vol.observed_voxel_count() == ora.observed_voxels() == vol.recount_observed_voxels()
    tris = backend.extract_mesh_cuda(vol)
    otris = ora.extract_mesh()
    assert tris.shape == otris.shape and tris.shape[0] > 1000
    assert np.array_equal(O.canonical_triangles(tris).view(np.uint32), O.canonical_triangles(otris).view(np.uint32))
    stats = (len(keys), vol.observed_voxel_count(), tris.shape[0])
    vol.close()
    ora.close()
    return stats


def test_small_orbit_configuration_bit_exact(env):
    backend, O, exp_impl = env
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=11, frames=64)
    K = sc.intrinsics
    assert (K.width, K.height, K.fx, K.fy, K.cx, K.cy) == (320, 240, 277.0, 277.0, 160.0, 120.0)
    assert (sc.voxel_size, sc.truncation, sc.hash_buckets) == (0.01, 0.04, 1 << 16)
    blocks, observed, triangles = _fuse_and_compare(backend, O, exp_impl, sc, list(range(0, 64, 4)),
                                                    hash_buckets=1 << 16, max_blocks=40000)
    assert blocks > 500 and observed > 100000


def test_room_configuration_first_frames_bit_exact(env):
    backend, O, exp_impl = env
    from voxelhashmt_gb300 import scenes
    sc = scenes.room_scene(seed=2, frames=4)
    K = sc.intrinsics
    assert (K.width, K.height, K.fx, K.fy) == (640, 480, 525.0, 525.0)
    assert (sc.voxel_size, sc.truncation) == (0.005, 0.02)
    blocks, observed, triangles = _fuse_and_compare(backend, O, exp_impl, sc, [0, 1, 2, 3],
                                                    hash_buckets=1 << 20, max_blocks=40000)
    assert blocks > 2000
