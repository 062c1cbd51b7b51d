"""GPU tests of the opt-in forms that trade bit parity for speed.

* truncation-band allocation (vh_algorithm.allocation_mode = 1): the blocks crossed by each pixel's
  [depth - trunc, depth + trunc] segment.  Its key set is a subset of the reference rule's (3 points x 27
  neighbours, the plain form) and contains every block the segment's three sample points fall in; it
  allocates and updates fewer blocks and voxels, and the fused surface stays as accurate as the plain form's
  (Chamfer to the analytic scene).
* fast-math depth filter and update pass (vh_algorithm.fast_math = 1): the same block set up to rare blocks at
  rounding distance from a block face, the same occupied layers almost everywhere, fields within a small
  tolerance of the exact form, and the same Chamfer.
* per-pixel normal map (vh_algorithm.normal_mode = 1): the map equals the reference's per-voxel normal
  evaluated at pixel centres (checked against the oracle's normal at integer coordinates), and the fused
  surface keeps the plain form's Chamfer.
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


def _sorted_keys(k):
    k = np.asarray(k, np.int32).reshape(-1, 3)
    return k[np.lexsort((k[:, 2], k[:, 1], k[:, 0]))]


def _fuse(backend, sc, frames, depths, stride=1, max_blocks=60000, **algo):
    from voxelhashmt_gb300 import _capi
    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 18, max_blocks=max_blocks,
                                algorithm=_capi.default_algorithm(**algo))
    bk = backend.TsdfIntegrationBackend("gpu")
    totals = {"visible_blocks": 0, "active_voxels": 0, "updated_voxels": 0}
    for f in frames:
        bk.integrate(vol, backend.DepthFrame(sc.intrinsics, depths[f]), sc.poses[f], stride)
        st = vol.frame_stats()
        for k in totals:
            totals[k] += st[k]
    return vol, totals


@pytest.fixture(scope="module")
def orbit_half():
    """The orbit scene (plane, sphere, box) at 160x120 (focal length halved), voxel 1 cm, truncation 4 cm,
    16 orbit frames."""
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=3, frames=16, width=160, height=120, fx=138.5, fy=138.5, cx=80.0, cy=60.0)
    sc.voxel_size, sc.truncation = 0.01, 0.04
    depths = [scenes.render_depth(sc, f) for f in range(16)]
    clean = [scenes.render_depth(sc, f, noise=False) for f in range(16)]
    return sc, depths, clean


def _block_of_points(sc, depth, f, stride):
    """Blocks of the three sample points of every sampled pixel (float64), with a flag for points more than
    1e-4 block from every block face (where float32 rounding cannot move them to a neighbour)."""
    K, P = sc.intrinsics, sc.poses[f]
    d = depth[::stride, ::stride].astype(np.float64)
    v, u = np.nonzero(d > 0)
    z = d[v, u]
    uu, vv = u * stride, v * stride
    pc = np.stack([(uu - K.cx) * z / K.fx, (vv - K.cy) * z / K.fy, z], axis=1)
    pw = pc @ np.asarray(P.R, np.float64).T + np.asarray(P.t, np.float64)
    ray = pw - np.asarray(P.t, np.float64)
    ray /= np.linalg.norm(ray, axis=1, keepdims=True)
    bws = 8 * sc.voxel_size
    out = []
    for q in (pw, pw - ray * sc.truncation, pw + ray * sc.truncation):
        g = q / bws
        frac = g - np.floor(g)
        safe = np.all((frac > 1e-4) & (frac < 1 - 1e-4), axis=1)
        out.append(np.floor(g[safe]).astype(np.int32))
    return np.unique(np.concatenate(out), axis=0)


@pytest.mark.parametrize("stride", [1, 2])
def test_band_keys_subset_of_reference_rule(backend, oracle_lib, small_orbit, stride):
    from voxelhashmt_gb300 import scenes
    O = oracle_lib
    sc = small_orbit
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN)
    for f in (0, 5, 13):
        d = scenes.render_depth(sc, f)
        vol, _ = _fuse(backend, sc, [f], {f: d}, stride=stride, max_blocks=8192, allocation_mode=1)
        got = _sorted_keys(backend.visible_block_keys(vol))
        vol.close()
        ref = O.collect_blocks(cfg, d, sc.intrinsics, sc.poses[f], sc.voxel_size, sc.truncation, stride)
        ref_set = {tuple(k) for k in ref}
        got_set = {tuple(k) for k in got}
        assert len(got_set) == got.shape[0], "duplicate keys in the visible list"
        assert got_set <= ref_set, "band block outside the reference rule's set"
        assert len(got_set) < len(ref_set)
        filtered = O.filter_depth(cfg, d, sc.intrinsics)  # allocation reads the filtered depth
        need = {tuple(k) for k in _block_of_points(sc, filtered, f, stride)}
        assert need <= got_set, "a block holding a sample point is missing from the band"
        # the exact compile walks the segments exactly as the oracle's statement of the band rule does
        want = O.collect_band_blocks(filtered, sc.intrinsics, sc.poses[f], sc.voxel_size, sc.truncation, stride)
        assert np.array_equal(got, want)


def _chamfer(backend, vol, sc, clean, frames):
    from voxelhashmt_gb300 import metrics
    tris = backend.extract_mesh_cuda(vol)
    pts = metrics.observed_surface_points(sc, frames, depth_maps=[clean[f] for f in frames], stride=2)
    return metrics.chamfer(tris, sc, pts), tris


def test_band_allocation_keeps_accuracy(backend, orbit_half):
    sc, depths, clean = orbit_half
    frames = list(range(16))
    plain, tp = _fuse(backend, sc, frames, depths)
    band, tb = _fuse(backend, sc, frames, depths, allocation_mode=1)
    cp, _ = _chamfer(backend, plain, sc, clean, frames)
    cb, _ = _chamfer(backend, band, sc, clean, frames)
    print("plain", tp, cp)
    print("band ", tb, cb)
    # The reference rule writes the observed surface into every voxel of the 27-block neighbourhoods that
    # projects in front of it; the band keeps the blocks within the truncation distance of the surface.
    assert tb["visible_blocks"] < 0.75 * tp["visible_blocks"], (tb, tp)
    assert tb["updated_voxels"] < tp["updated_voxels"], (tb, tp)
    assert cb["chamfer_mm"] <= cp["chamfer_mm"] * 1.05 + 0.05, (cb, cp)
    plain.close()
    band.close()


def test_fast_math_matches_exact(backend, orbit_half):
    """Fast-math vs exact depth filter and update pass on the same frames.  Block keys agree to 0.1% (the
    allocation is exact in both, but reads the filtered depth, whose last bits differ, so a point within a
    rounding of a block face can land in the neighbouring block).  Where both forms hold a layer of a common
    block: weights within 1e-3 relative and surface coordinates / plane offsets within 5e-3 voxel for 99.9%
    of layers.  The coordinates are world metres of magnitude ~1, so
    5e-3 voxel (5e-5 m at 1 cm) is a few float32 ulp: the last-bit differences of the approximate division,
    square root and exponential, compounded over frames; rare voxels where a rounding flips a layer-match
    decision account for the rest.  Layer occupancy agrees on 99.9% of voxel bins, and the Chamfer distance
    to the analytic surface agrees within 2%."""
    sc, depths, clean = orbit_half
    frames = list(range(0, 16, 2))
    from oracle import oracle as O
    ex, te = _fuse(backend, sc, frames, depths)
    fa, tf = _fuse(backend, sc, frames, depths, fast_math=1)
    ke, ve = O.sort_blocks(*ex.export_blocks())
    kf, vf = O.sort_blocks(*fa.export_blocks())
    ie = {tuple(k): i for i, k in enumerate(ke.tolist())}
    common = [(ie[k], j) for j, k in enumerate(map(tuple, kf.tolist())) if k in ie]
    assert len(common) >= 0.999 * max(len(ke), len(kf)), (len(common), len(ke), len(kf))
    ce_idx = np.array([a for a, _ in common])
    cf_idx = np.array([b for _, b in common])
    e = ve[ce_idx].view(np.float32).reshape(-1, 4)
    g = vf[cf_idx].view(np.float32).reshape(-1, 4)
    occ_e, occ_f = e[:, 0] > 0, g[:, 0] > 0
    assert occ_e.sum() > 10000
    assert np.mean(occ_e == occ_f) >= 0.999
    both = occ_e & occ_f
    w_err = np.abs(g[both, 0] - e[both, 0]) / e[both, 0]
    assert np.quantile(w_err, 0.999) <= 1e-3, float(np.quantile(w_err, 0.999))
    for col in (1, 2):
        c_err = np.abs(g[both, col].astype(np.float64) - e[both, col]) / sc.voxel_size
        assert np.quantile(c_err, 0.999) <= 5e-3, (col, float(np.quantile(c_err, 0.999)))
    ce, _ = _chamfer(backend, ex, sc, clean, frames)
    cf, _ = _chamfer(backend, fa, sc, clean, frames)
    print("exact", ce)
    print("fast ", cf)
    assert abs(cf["chamfer_mm"] - ce["chamfer_mm"]) <= 0.02 * ce["chamfer_mm"], (cf, ce)
    ex.close()
    fa.close()


def test_normal_map_keeps_accuracy(backend, orbit_half):
    sc, depths, clean = orbit_half
    frames = list(range(16))
    plain, tp = _fuse(backend, sc, frames, depths)
    mapped, tm = _fuse(backend, sc, frames, depths, normal_mode=1)
    chosen, tc = _fuse(backend, sc, frames, depths, allocation_mode=1, fast_math=1, normal_mode=1)
    cp, _ = _chamfer(backend, plain, sc, clean, frames)
    cm, _ = _chamfer(backend, mapped, sc, clean, frames)
    cc, _ = _chamfer(backend, chosen, sc, clean, frames)
    print("plain ", tp, cp)
    print("map   ", tm, cm)
    print("chosen", tc, cc)
    # the map form visits the same voxels as the plain form (same allocation, same prefix test)
    assert tm["active_voxels"] == tp["active_voxels"]
    assert cm["chamfer_mm"] <= cp["chamfer_mm"] * 1.05 + 0.05, (cm, cp)
    assert cc["chamfer_mm"] <= cp["chamfer_mm"] * 1.05 + 0.05, (cc, cp)
    for v in (plain, mapped, chosen):
        v.close()


@pytest.mark.parametrize("fast_math", [0, 1])
def test_fused_update_visits_every_active_voxel(backend, orbit_half, fast_math):
    """Every launch shape of the fused layer update (normal_mode 1) visits the voxels that the classify pass of
    the per-voxel-normal form (normal_mode 0) visits: the same prefix test on the same allocation.  The
    active-voxel totals agree exactly in the exact compile and to 1e-5 in the fast-math compile, where the
    projection's approximate division can move a voxel across the image border or the truncation limit.  A
    kernel that dropped queued survivors falls short by whole warps: at least 1/16 of a chunk."""
    sc, depths, _ = orbit_half
    frames = list(range(8))
    ref, tr = _fuse(backend, sc, frames, depths, allocation_mode=1, fast_math=fast_math)
    ref.close()
    assert tr["active_voxels"] > 100000
    for variant in range(6):
        vol, t = _fuse(backend, sc, frames, depths, allocation_mode=1, fast_math=fast_math, normal_mode=1,
                       autotune=0, launch_variant=variant)
        assert vol.observed_voxel_count() == vol.recount_observed_voxels(), variant
        vol.close()
        if fast_math == 0:
            assert t["active_voxels"] == tr["active_voxels"], (variant, t, tr)
        else:
            assert abs(t["active_voxels"] - tr["active_voxels"]) <= 1e-5 * tr["active_voxels"], (variant, t, tr)


def test_opt_in_form_empty_frame_and_full_pool(backend, small_orbit):
    """The opt-in form (band allocation, normal map, fast math, FP16 bins) on the edge cases the plain form is
    tested on.  An all-zero frame allocates and updates nothing: the fused update then has no chunk.  A pool
    too small for the frame reports VH_ERR_POOL_FULL and keeps the blocks that fit; the visible entries left
    without a pool block are skipped by the normal-map pass and the fused update, and the counters stay
    consistent with a recount."""
    from voxelhashmt_gb300 import _capi, scenes
    sc = small_orbit
    algo = _capi.default_algorithm(allocation_mode=1, normal_mode=1, fast_math=1)
    d = scenes.render_depth(sc, 0)
    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 16, max_blocks=8192, layer_format=1,
                                algorithm=algo)
    z = np.zeros((sc.intrinsics.height, sc.intrinsics.width), np.float32)
    backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, z), sc.poses[0])
    st = vol.frame_stats()
    assert st["visible_blocks"] == 0 and st["active_voxels"] == 0 and st["updated_voxels"] == 0
    assert vol.block_count() == 0 and vol.observed_voxel_count() == 0
    assert backend.extract_mesh_cuda(vol).shape == (0, 9)
    backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[0])
    assert vol.block_count() > 0 and vol.observed_voxel_count() > 0
    assert vol.observed_voxel_count() == vol.recount_observed_voxels()
    vol.close()
    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 16, max_blocks=16, layer_format=1,
                                algorithm=algo)
    with pytest.raises(_capi.VhError) as e:
        backend.integrate_depth_frame_cuda(vol, backend.DepthFrame(sc.intrinsics, d), sc.poses[0])
    assert e.value.status == _capi.VH_ERR_POOL_FULL
    assert vol.block_count() == 16
    n = vol.observed_voxel_count()
    assert 0 < n <= 16 * 512 and n == vol.recount_observed_voxels()
    vol.close()


@pytest.mark.parametrize("fast_math", [0, 1])
def test_pixel_normal_map_matches_reference_normal(backend, oracle_lib, fast_math):
    """The map at pixel centres against the oracle's estimateSurfaceNormalCamera at integer coordinates:
    bit-identical in the exact form; validity identical and directions within 1e-3 rad (0.06 degree) for
    99.9% of pixels in the fast form, whose hardware exponential has an error that grows with the argument
    (the angular and range Gaussians of the bilateral weights take arguments up to ~100)."""
    import ctypes as C
    from voxelhashmt_gb300 import _capi, scenes
    O = oracle_lib
    sc = scenes.orbit_scene(seed=9, frames=4, width=97, height=61, fx=84.0, fy=84.0, cx=48.5, cy=30.5)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, max_blocks=1,
                                algorithm=_capi.default_algorithm(fast_math=fast_math, normal_mode=1))
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN)
    for f in (0, 2):
        d = O.filter_depth(cfg, scenes.render_depth(sc, f), sc.intrinsics)
        dd = torch.from_numpy(d).cuda()
        out = torch.zeros((d.size, 4), dtype=torch.float32, device="cuda")
        Kc = _capi.intrinsics(sc.intrinsics)
        _capi.check(_capi.lib().vh_pixel_normals(vol.handle, C.c_void_p(dd.data_ptr()), C.c_void_p(out.data_ptr()),
                                                 C.byref(Kc), None), vol.handle)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(d.shape + (4,))
        want_n, want_ok = O.pixel_normals(cfg, d, sc.intrinsics)
        assert np.array_equal(got[..., 3] > 0, want_ok > 0)
        assert want_ok.sum() > 0.5 * d.size
        ok = want_ok > 0
        if fast_math == 0:
            assert np.array_equal(got[ok, :3].view(np.uint32), want_n[ok].view(np.uint32))
        else:
            cosang = np.clip(np.sum(got[ok, :3].astype(np.float64) * want_n[ok], axis=1), -1.0, 1.0)
            assert np.quantile(np.arccos(cosang), 0.999) <= 1e-3
    vol.close()


@pytest.mark.parametrize("chosen", [False, True])
def test_fp16_storage_matches_fp32(backend, orbit_half, chosen):
    """FP16 layer storage (vh_params.layer_format 1) against FP32 storage, same frames, same algorithm.
    Stated per-field errors, for layers observed in both, at the 99th percentile: weight within 1e-3
    relative (binary16 rounding of the accumulated weight, 2^-11 per update); surface coordinate and plane
    offset within 0.03 voxel (binary16 step of the voxel-relative value, <= 1/64 voxel below 16 voxels, plus
    the slightly different blending weights).  Beyond that percentile the differences are layer-assignment
    flips: a rounded coordinate crosses the merge tolerance or the layer order, and the observation lands
    in another layer of the bin, so both the weight and the coordinates of that slot differ by whole
    observations; at most 1% of layers.  Block keys identical, layer occupancy equal on 99.9% of bins,
    incremental observed count equal to the recount, Chamfer within 2% of the FP32 form's."""
    sc, depths, clean = orbit_half
    frames = list(range(0, 16, 2))
    from oracle import oracle as O
    algo = dict(allocation_mode=1, fast_math=1, normal_mode=1) if chosen else {}
    from voxelhashmt_gb300 import _capi
    vols = []
    for fmt in (0, 1):
        vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 18, max_blocks=60000,
                                    algorithm=_capi.default_algorithm(**algo), layer_format=fmt)
        bk = backend.TsdfIntegrationBackend("gpu")
        for f in frames:
            bk.integrate(vol, backend.DepthFrame(sc.intrinsics, depths[f]), sc.poses[f], 1)
        vols.append(vol)
    k32, v32 = O.sort_blocks(*vols[0].export_blocks())
    k16, v16 = O.sort_blocks(*vols[1].export_blocks())
    assert np.array_equal(k32, k16)
    a = v32.view(np.float32).reshape(-1, 4)
    b = v16.view(np.float32).reshape(-1, 4)
    occ_a, occ_b = a[:, 0] > 0, b[:, 0] > 0
    assert occ_a.sum() > 10000
    assert np.mean(occ_a == occ_b) >= 0.999
    both = occ_a & occ_b
    w_err = np.abs(b[both, 0] - a[both, 0]) / a[both, 0]
    errs = {"weight_rel": w_err}
    for col, name in ((1, "surface_coord_vox"), (2, "plane_offset_vox")):
        errs[name] = np.abs(b[both, col].astype(np.float64) - a[both, col]) / sc.voxel_size
    for name, e in errs.items():
        print("fp16-vs-fp32 %-18s q50 %.3g q90 %.3g q99 %.3g q999 %.3g max %.3g" % (
            name, *(float(np.quantile(e, q)) for q in (0.5, 0.9, 0.99, 0.999)), float(e.max())))
    assert np.quantile(w_err, 0.99) <= 1e-3, float(np.quantile(w_err, 0.99))
    for name in ("surface_coord_vox", "plane_offset_vox"):
        assert np.quantile(errs[name], 0.99) <= 0.03, (name, float(np.quantile(errs[name], 0.99)))
    flipped = (w_err > 1e-2) | (errs["surface_coord_vox"] > 0.25) | (errs["plane_offset_vox"] > 0.25)
    print("fp16-vs-fp32 layer-assignment flips: %.4f%% of layers" % (100.0 * float(np.mean(flipped))))
    assert np.mean(flipped) <= 0.01
    assert vols[1].observed_voxel_count() == vols[1].recount_observed_voxels()
    c32, _ = _chamfer(backend, vols[0], sc, clean, frames)
    c16, _ = _chamfer(backend, vols[1], sc, clean, frames)
    print("fp32", c32)
    print("fp16", c16)
    assert abs(c16["chamfer_mm"] - c32["chamfer_mm"]) <= 0.02 * c32["chamfer_mm"], (c16, c32)
    # checkpoint round trip through the reference FP32 layout into a fresh FP16 volume
    keys, vox = vols[1].export_blocks()
    fresh = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 18, max_blocks=60000,
                                  layer_format=1)
    fresh.import_blocks(keys, vox)
    k2, v2 = O.sort_blocks(*fresh.export_blocks())
    assert np.array_equal(k2, k16)
    x2 = v2.view(np.float32).reshape(-1, 4)
    assert np.array_equal(x2[:, 0] > 0, b[:, 0] > 0)
    assert np.array_equal(x2[:, 3].view(np.uint32), b[:, 3].view(np.uint32))
    assert np.array_equal(x2[:, 0], b[:, 0])
    assert np.max(np.abs(x2[:, 1:3].astype(np.float64) - b[:, 1:3])) <= 1e-3 * sc.voxel_size
    assert fresh.observed_voxel_count() == vols[1].observed_voxel_count()
    for v in vols + [fresh]:
        v.close()


@pytest.mark.parametrize("fast_math", [0, 1])
def test_autotuned_launch_shapes_give_identical_volumes(backend, orbit_half, fast_math):
    """The autotuner cycles the layer update through its launch shapes on the first frames; every shape runs
    the same per-voxel update.  In the exact compile (no contraction, IEEE division and square root) the
    volume is bit-identical to one fused with a fixed shape.  In the fast-math compile each shape is a
    separate instantiation whose multiply-add contraction the compiler decides on its own, so fields may
    differ in the last bits: identical keys and occupancy on 99.9% of bins, fields within 1e-3 voxel
    (99.9%)."""
    sc, depths, _ = orbit_half
    # 68 frames: 24 before tuning, 10 shapes x 4 rounds of tuning, then the kept shape
    frames = list(range(16)) * 4 + list(range(4))
    from oracle import oracle as O
    algo = dict(allocation_mode=1, fast_math=fast_math, normal_mode=1)
    tuned, _ = _fuse(backend, sc, frames, depths, **algo)
    fixed, _ = _fuse(backend, sc, frames, depths, autotune=0, **algo)
    res = tuned.autotune_result()
    print("autotune", fast_math, res)
    assert res["variant"] >= 0 and res["threads_per_cta"] in (64, 128, 256, 512) and res["ms"] > 0
    assert fixed.autotune_result()["variant"] == -1
    k1, v1 = O.sort_blocks(*tuned.export_blocks())
    k2, v2 = O.sort_blocks(*fixed.export_blocks())
    assert np.array_equal(k1, k2)
    print("differing words", int(np.sum(v1 != v2)), "of", v1.size)
    if fast_math == 0:
        assert np.array_equal(v1, v2)
        assert tuned.observed_voxel_count() == fixed.observed_voxel_count()
    else:
        a = v1.view(np.float32).reshape(-1, 4)
        b = v2.view(np.float32).reshape(-1, 4)
        assert np.mean((a[:, 0] > 0) == (b[:, 0] > 0)) >= 0.999
        both = (a[:, 0] > 0) & (b[:, 0] > 0)
        for col in (1, 2):
            e = np.abs(a[both, col].astype(np.float64) - b[both, col]) / sc.voxel_size
            assert np.quantile(e, 0.999) <= 1e-3, (col, float(np.quantile(e, 0.999)))
    tuned.close()
    fixed.close()


@pytest.mark.parametrize("scene", ["small", "half"])
@pytest.mark.parametrize("alloc,fp16", [(1, 1), (0, 1), (1, 0), (0, 0)])
def test_opt_in_switches_bit_exact_in_the_exact_compile(backend, oracle_lib, small_orbit, orbit_half, scene, alloc,
                                                        fp16):
    """The headline form's switches without fast math -- per-pixel normal map (normal_mode 1), truncation-band
    allocation (allocation_mode 1) and FP16 bins (layer_format 1) -- against the oracle's restatement of the
    same switches (vo_config.alloc_mode / normal_mode / layer_format): the visible block count of every frame,
    every voxel word as exported (FP16 bins decoded), the observed-voxel count and the marching-cubes soup are
    bit-identical.  Only the fast-math compile of the form is left to the statistical tests above."""
    O = oracle_lib
    from voxelhashmt_gb300 import _capi, scenes
    if scene == "small":
        sc, frames = small_orbit, [0, 5, 10, 15, 20]
        depths = {f: scenes.render_depth(sc, f) for f in frames}
    else:
        (sc, dl, _), frames = orbit_half, [0, 3, 6, 9, 12, 15]
        depths = {f: dl[f] for f in frames}
    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=1 << 18, max_blocks=60000,
                                algorithm=_capi.default_algorithm(allocation_mode=alloc, normal_mode=1, fast_math=0,
                                                                  autotune=0),
                                layer_format=fp16)
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN, threads=8, alloc_mode=alloc, normal_mode=1, layer_format=fp16)
    ora = O.Volume(cfg, sc.voxel_size, sc.truncation)
    bk = backend.TsdfIntegrationBackend("gpu")
    for f in frames:
        bk.integrate(vol, backend.DepthFrame(sc.intrinsics, depths[f]), sc.poses[f], 1)
        n = ora.integrate(depths[f], sc.intrinsics, sc.poses[f])
        assert vol.frame_stats()["visible_blocks"] == n, f
    gk, gv = O.sort_blocks(*vol.export_blocks())
    ok, ov = O.sort_blocks(*ora.blocks())
    assert np.array_equal(gk, ok)
    assert np.array_equal(gv.reshape(len(gk), -1), ov.view(np.uint32).reshape(len(ok), -1))
    assert vol.observed_voxel_count() == ora.observed_voxels() == vol.recount_observed_voxels()
    tris = backend.extract_mesh_cuda(vol)
    assert tris.shape[0] > 1000
    assert np.array_equal(O.canonical_triangles(tris).view(np.uint32),
                          O.canonical_triangles(ora.extract_mesh()).view(np.uint32))
    vol.close()
    ora.close()

