"""GPU tests of the multi-scene batch (vh_batch_*): many volumes of different resolutions, voxel sizes, storage
formats and frame counts fused in shared work-queue kernels: launched one by one, captured in a CUDA graph, and as
one persistent cooperative launch per step.

In the exact compile (fast_math 0) every scene's volume is bit-identical to fusing that scene alone with the
same settings; the fast-math batch with and without the graph are bit-identical to each other, and its
surfaces keep the exact batch's Chamfer distance.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend(product_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxelhashmt_gb300 import backend as b
    return b


def _scenes():
    from voxelhashmt_gb300 import scenes
    out = []
    specs = [(64, 48, 0.02, 0), (160, 120, 0.01, 1), (97, 61, 0.015, 0), (128, 96, 0.008, 1), (40, 30, 0.02, 1),
             (200, 150, 0.012, 0)]
    for k, (w, h, vs, fmt) in enumerate(specs):
        sc = scenes.orbit_scene(seed=20 + k, frames=12, width=w, height=h, fx=0.866 * w, fy=0.866 * w, cx=w / 2,
                                cy=h / 2)
        sc.voxel_size, sc.truncation = vs, 3 * vs
        out.append((sc, fmt, [scenes.render_depth(sc, f) for f in range(12)]))
    return out


def _volume(backend, sc, fmt, fast):
    from voxelhashmt_gb300 import _capi
    return backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 16, max_blocks=20000, layer_format=fmt,
                                 algorithm=_capi.default_algorithm(allocation_mode=1, normal_mode=1, fast_math=fast))


def _run_batch(backend, scs, fast, use_graph, steps):
    vols = [_volume(backend, sc, fmt, fast) for sc, fmt, _ in scs]
    batch = backend.VolumeBatch(vols, use_graph=use_graph)
    dev = [[torch.from_numpy(d).cuda() for d in deps] for _, _, deps in scs]
    for step in range(steps):
        # ragged: scene k has 12 - k frames and starts at step k // 2
        depths, Ks, Ps = [], [], []
        for k, (sc, _, _) in enumerate(scs):
            f = step - k // 2
            on = 0 <= f < 12 - k
            depths.append(dev[k][f].view(-1) if on else None)
            Ks.append(sc.intrinsics)
            Ps.append(sc.poses[f] if on else sc.poses[0])
        batch.integrate(depths, Ks, Ps)
    torch.cuda.synchronize()
    for v in vols:
        v.synchronize()
    batch.close()
    return vols


def _run_alone(backend, scs, fast):
    vols = []
    bk = backend.TsdfIntegrationBackend("gpu")
    for k, (sc, fmt, deps) in enumerate(scs):
        v = _volume(backend, sc, fmt, fast)
        for f in range(12 - k):
            bk.integrate(v, backend.DepthFrame(sc.intrinsics, torch.from_numpy(deps[f]).cuda().view(-1)), sc.poses[f])
        vols.append(v)
    return vols


@pytest.mark.parametrize("use_graph", [False, True, "persistent"])
def test_batch_equals_scenes_alone_exact(backend, oracle_lib, use_graph):
    O = oracle_lib
    scs = _scenes()
    steps = 12 + len(scs) // 2
    batched = _run_batch(backend, scs, 0, use_graph, steps)
    alone = _run_alone(backend, scs, 0)
    for k, (a, b) in enumerate(zip(batched, alone)):
        ka, va = O.sort_blocks(*a.export_blocks())
        kb, vb = O.sort_blocks(*b.export_blocks())
        assert ka.shape[0] > 0
        assert np.array_equal(ka, kb), k
        assert np.array_equal(va, vb), k
        assert a.observed_voxel_count() == b.observed_voxel_count() == a.recount_observed_voxels()
        assert a.frame_stats()["updated_voxels"] == b.frame_stats()["updated_voxels"]
    for v in batched + alone:
        v.close()


def test_batch_fast_math_graph_and_stream_agree(backend, oracle_lib):
    O = oracle_lib
    from voxelhashmt_gb300 import metrics
    scs = _scenes()
    steps = 12 + len(scs) // 2
    g = _run_batch(backend, scs, 1, True, steps)
    s = _run_batch(backend, scs, 1, False, steps)
    e = _run_batch(backend, scs, 0, True, steps)
    alone = _run_alone(backend, scs, 1)
    for k, (a, b, c) in enumerate(zip(g, s, e)):
        ka, va = O.sort_blocks(*a.export_blocks())
        kb, vb = O.sort_blocks(*b.export_blocks())
        assert np.array_equal(ka, kb) and np.array_equal(va, vb), k
        # every queued survivor is updated and counted: the same observed voxels as the scene fused alone in
        # the fast-math form (up to rounding at the band and image edges), and the counter equals a recount
        n_alone = alone[k].observed_voxel_count()
        assert a.observed_voxel_count() == a.recount_observed_voxels(), k
        assert abs(a.observed_voxel_count() - n_alone) <= 1e-3 * n_alone + 10, (k, a.observed_voxel_count(), n_alone)
        sc = scs[k][0]
        frames = list(range(12 - k))
        pts = metrics.observed_surface_points(sc, frames, stride=2)
        qa = metrics.chamfer(backend.extract_mesh_cuda(a), sc, pts)
        qc = metrics.chamfer(backend.extract_mesh_cuda(c), sc, pts)
        assert abs(qa["chamfer_mm"] - qc["chamfer_mm"]) <= 0.03 * qc["chamfer_mm"] + 0.05, (k, qa, qc)
    for v in g + s + e + alone:
        v.close()


@pytest.mark.parametrize("use_graph", [False, True, "persistent"])
def test_batch_scene_with_full_pool_does_not_affect_the_others(backend, oracle_lib, use_graph):
    """One scene of a batch runs out of pool blocks: its error surfaces on its own volume (vh_synchronize
    reports VH_ERR_POOL_FULL, the blocks that fit are kept and consistently counted), its visible entries
    without a pool block are skipped by the normal-map and update kernels, and the other scene fuses exactly
    as it does alone (exact compile)."""
    O = oracle_lib
    from voxelhashmt_gb300 import _capi
    scs = _scenes()[:2]
    (sc0, fmt0, dep0), (sc1, fmt1, dep1) = scs
    small = backend.VoxelHashTSDF(sc0.voxel_size, sc0.truncation, hash_buckets=1 << 16, max_blocks=16,
                                  layer_format=fmt0,
                                  algorithm=_capi.default_algorithm(allocation_mode=1, normal_mode=1, fast_math=0))
    other = _volume(backend, sc1, fmt1, 0)
    batch = backend.VolumeBatch([small, other], use_graph=use_graph)
    for f in range(6):
        batch.integrate([torch.from_numpy(dep0[f]).cuda().view(-1), torch.from_numpy(dep1[f]).cuda().view(-1)],
                        [sc0.intrinsics, sc1.intrinsics], [sc0.poses[f], sc1.poses[f]])
    torch.cuda.synchronize()
    with pytest.raises(_capi.VhError) as e:
        small.synchronize()
    assert e.value.status == _capi.VH_ERR_POOL_FULL
    assert small.block_count() == 16
    n = small.observed_voxel_count()
    assert 0 < n <= 16 * 512 and n == small.recount_observed_voxels()
    other.synchronize()
    alone = _volume(backend, sc1, fmt1, 0)
    bk = backend.TsdfIntegrationBackend("gpu")
    for f in range(6):
        bk.integrate(alone, backend.DepthFrame(sc1.intrinsics, torch.from_numpy(dep1[f]).cuda().view(-1)), sc1.poses[f])
    ka, va = O.sort_blocks(*other.export_blocks())
    kb, vb = O.sort_blocks(*alone.export_blocks())
    assert ka.shape[0] > 0 and np.array_equal(ka, kb) and np.array_equal(va, vb)
    batch.close()
    for v in (small, other, alone):
        v.close()

