"""CPU tests of the parity oracle: pinned against the reference's own outputs.

* against the committed fixtures in tests/golden/ (made by tests/golden/make_golden.py from the reference
  build): filtered depth, allocated block keys, every voxel byte (SHA-256), observed-voxel count and the
  triangle soup, for the reference CUDA path (emulated on the host) and the reference CPU path;
* against the live reference build (oracle/_ref/libref.so) where the reference tree is present, on more
  frames and strides;
* known-answer tests of the key hash, key packing, octahedral packing and the observation weight;
* the product's exponential against float64 exp;
* the restatement against the FP64 transcription (the same source in double arithmetic), with stated
  tolerances.
"""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


@pytest.fixture(scope="module")
def golden_scene():
    from voxelhashmt_gb300 import scenes
    g = np.load(os.path.join(GOLDEN, "golden_scene.npz"))
    w, h, fx, fy, cx, cy = g["intrinsics"]
    K = scenes.Intrinsics(int(w), int(h), float(fx), float(fy), float(cx), float(cy))
    poses = [scenes.Pose(p[:9].reshape(3, 3).copy(), p[9:].copy()) for p in g["poses"]]
    return {"depth": g["depth"], "K": K, "poses": poses, "vs": float(g["voxel_size"]), "trunc": float(g["truncation"])}


@pytest.mark.parametrize("exp_name", ["libm", "own"])
@pytest.mark.parametrize("flavor_name", ["gpu", "cpu"])
def test_oracle_matches_reference_fixtures(O, golden_scene, flavor_name, exp_name):
    """With the C library's expf, and with its restatement (which makes the check independent of the host's C
    library), the oracle reproduces the reference's own outputs bit for bit."""
    gs = golden_scene
    ref = np.load(os.path.join(GOLDEN, "golden_%s.npz" % flavor_name))
    flavor = O.FLAVOR_REF_GPU if flavor_name == "gpu" else O.FLAVOR_REF_CPU
    cfg = O.config(flavor, O.EXP_LIBM if exp_name == "libm" else O.EXP_OWN, threads=4)
    K = gs["K"]
    d0 = gs["depth"][0]
    assert np.array_equal(_bits(O.filter_depth(cfg, d0, K)), _bits(ref["filtered0"]))
    for stride in (1, 2):
        keys = O.collect_blocks(cfg, d0, K, gs["poses"][0], gs["vs"], gs["trunc"], stride)
        assert np.array_equal(keys, ref["keys_stride%d" % stride])
    vol = O.Volume(cfg, gs["vs"], gs["trunc"])
    for d, P in zip(gs["depth"], gs["poses"]):
        vol.integrate(d, K, P)
    keys, vox = O.sort_blocks(*vol.blocks())
    assert np.array_equal(keys, ref["block_keys"])
    assert vol.observed_voxels() == int(ref["observed_voxels"])
    assert hashlib.sha256(np.ascontiguousarray(vox).view(np.uint8).tobytes()).hexdigest() == str(ref["voxel_sha256"])
    for k, v in zip(ref["fullest_keys"], ref["fullest_voxels"]):
        i = int(np.nonzero((keys == k).all(axis=1))[0][0])
        assert np.array_equal(vox[i].view(np.uint32), v)
    tris = O.canonical_triangles(vol.extract_mesh())
    assert np.array_equal(_bits(tris), _bits(ref["triangles"]))
    vol.close()


def test_known_answers(O):
    import ctypes as C
    kat = np.load(os.path.join(GOLDEN, "golden_kat.npz"))
    L = O.lib()
    for k, h, pk, ok in zip(kat["keys"], kat["hashes"], kat["packed"], kat["packable"]):
        assert L.vo_hash_block_key(*map(int, k)) == int(h)
        p = C.c_uint64()
        assert L.vo_pack_block_key(*map(int, k), C.byref(p)) == int(ok)
        if ok:
            assert p.value == int(pk)
    fp = C.POINTER(C.c_float)
    for n, pg, pc in zip(kat["normals"], kat["pack_gpu"], kat["pack_cpu"]):
        n = np.ascontiguousarray(n, np.float32)
        assert O.lib().vo_pack_normal(O.FLAVOR_REF_GPU, n.ctypes.data_as(fp)) == int(pg)
        assert O.lib().vo_pack_normal(O.FLAVOR_REF_CPU, n.ctypes.data_as(fp)) == int(pc)
    out = np.zeros(3, np.float32)
    for name, flavor, mesh in (("unpack_gpu", O.FLAVOR_REF_GPU, 0), ("unpack_gpu_mesh", O.FLAVOR_REF_GPU, 1),
                               ("unpack_cpu", O.FLAVOR_REF_CPU, 0)):
        for code, want in zip(kat["codes"], kat[name]):
            O.lib().vo_unpack_normal(flavor, mesh, int(code), out.ctypes.data_as(fp))
            assert np.array_equal(_bits(out), _bits(want)), (name, int(code))
    cfg = O.config(O.FLAVOR_REF_GPU)
    for a, w in zip(kat["weight_args"], kat["weights"]):
        got = O.lib().vo_observation_weight(C.byref(cfg), *map(float, a))
        assert np.float32(got).view(np.uint32) == np.float32(w).view(np.uint32)


def _glibc_expf_host():
    import platform
    lib, ver = platform.libc_ver()
    try:
        major, minor = (int(v) for v in ver.split(".")[:2])
    except ValueError:
        return False
    return lib == "glibc" and (major, minor) >= (2, 28)


@pytest.mark.skipif(not _glibc_expf_host(), reason="the restated expf is the GNU C library's (glibc >= 2.28)")
def test_own_exp_is_the_c_library_expf(O):
    """vo_expf_own (restated in the oracle and, identically, on the device as vh_expf) returns the C library's
    expf for every float argument: all non-positive floats (the path's arguments, -sq / (2 sigma^2)) and all
    positive ones, exhaustively."""
    threads = max(os.cpu_count() or 1, 1)
    for first in (0x80000000, 0x00000000):  # -0 ... -inf, then +0 ... +inf
        n, bad = O.expf_compare_libm(first, 0x7F800001, threads=threads)
        assert n == 0, "%d differing arguments, the first %08x" % (n, bad)
    L = O.lib()
    assert L.vo_expf_own(0.0) == 1.0 and L.vo_expf_own(-0.0) == 1.0
    assert L.vo_expf_own(-200.0) == 0.0 and L.vo_expf_own(float("-inf")) == 0.0
    assert L.vo_expf_own(100.0) == float("inf") and np.isnan(L.vo_expf_own(float("nan")))


def test_own_exp_accuracy(O):
    """vo_expf_own is within 0.51 ulp of exp (float64 reference) over the arguments the path uses."""
    xs = np.concatenate([-np.logspace(-8, np.log10(103.0), 20000), np.linspace(-20.0, 0.0, 20001),
                         np.linspace(0.0, 80.0, 2001)]).astype(np.float32)
    got = O.expf_array(xs)
    want = np.exp(xs.astype(np.float64))
    normal = want > np.float64(np.finfo(np.float32).tiny)
    ulp = np.spacing(want[normal].astype(np.float32)).astype(np.float64)
    err = np.abs(got[normal].astype(np.float64) - want[normal]) / ulp
    assert err.max() <= 0.51, float(err.max())


ref_only = pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libref.so")),
                              reason="reference build (oracle/_ref) not present on this machine")


@ref_only
@pytest.mark.parametrize("gpu", [True, False])
def test_oracle_matches_live_reference(O, gpu):
    """Several frames, strides 1 and 3, both flavours, against the reference compiled from its sources."""
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=77, frames=10, width=56, height=40, fx=48.5, fy=48.5, cx=27.5, cy=19.5)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    K = sc.intrinsics
    cfg = O.config(O.FLAVOR_REF_GPU if gpu else O.FLAVOR_REF_CPU, O.EXP_LIBM, threads=4)
    for f, stride in ((1, 1), (6, 3)):
        d = scenes.render_depth(sc, f)
        assert np.array_equal(_bits(O.filter_depth(cfg, d, K)), _bits(O.ref_filter(d, K, gpu)))
        ko = O.collect_blocks(cfg, d, K, sc.poses[f], sc.voxel_size, sc.truncation, stride)
        kr = O.ref_collect(d, K, sc.poses[f], sc.voxel_size, sc.truncation, stride, gpu)
        assert np.array_equal(ko, kr)
    vo = O.Volume(cfg, sc.voxel_size, sc.truncation)
    vr = O.RefVolume(gpu, sc.voxel_size, sc.truncation)
    for f in (0, 3, 7):
        d = scenes.render_depth(sc, f)
        vo.integrate(d, K, sc.poses[f], 2)
        vr.integrate(d, K, sc.poses[f], 2)
    ko, xo = O.sort_blocks(*vo.blocks())
    kr, xr = O.sort_blocks(*vr.blocks())
    assert np.array_equal(ko, kr)
    assert np.array_equal(xo.view(np.uint32), xr.view(np.uint32))
    assert vo.observed_voxels() == vr.observed_voxels()
    assert np.array_equal(_bits(O.canonical_triangles(vo.extract_mesh())),
                          _bits(O.canonical_triangles(vr.extract_mesh())))
    vr.close()
    vo.close()


@ref_only
def test_mc_tables_match_reference_header():
    import re
    from oracle import build as ob
    ref = os.path.join(ob.REFERENCE, "include", "tsdfmc", "marching_cubes_tables.h")
    if not os.path.exists(ref):
        pytest.skip("reference header not present")
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen", os.path.join(os.path.dirname(HERE), "oracle", "gen_mc_tables.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    edge, tri = gen.parse_reference(ref)
    text = open(os.path.join(os.path.dirname(HERE), "voxelhashmt_gb300", "csrc", "vh_mc_tables.h")).read()
    body_e = text[text.index("vh_mc_edge_table[256] = {"):text.index("};")]
    ours_e = [int(x) for x in re.findall(r"-?\d+", body_e.split("{", 1)[1])]
    body_t = text[text.index("vh_mc_tri_table[256][16] = {"):]
    ours_t = [int(x) for x in re.findall(r"-?\d+", body_t.split("= {", 1)[1].split("};", 1)[0])]
    assert ours_e == edge
    assert ours_t == [v for row in tri for v in row]


def test_oracle_parallel_equals_serial(O):
    """threads > 1 (the CPU baseline's setting) gives the same volume as the literal serial order."""
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=5, frames=4, width=40, height=30, fx=34.6, fy=34.6, cx=20.0, cy=15.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    res = []
    for threads in (1, 4):
        v = O.Volume(O.config(O.FLAVOR_REF_CPU, O.EXP_LIBM, threads=threads), sc.voxel_size, sc.truncation)
        for f in range(2):
            v.integrate(scenes.render_depth(sc, f), sc.intrinsics, sc.poses[f])
        k, x = O.sort_blocks(*v.blocks())
        res.append((k, x.view(np.uint32), O.canonical_triangles(v.extract_mesh())))
        v.close()
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    assert np.array_equal(_bits(res[0][2]), _bits(res[1][2]))


def test_band_rule_known_answers(O):
    """The truncation-band rule on single rays whose crossings are known by hand."""
    from voxelhashmt_gb300 import scenes
    K = scenes.Intrinsics(1, 1, 1.0, 1.0, 0.0, 0.0)
    eye = scenes.Pose(np.eye(3, dtype=np.float32), np.zeros(3, np.float32))
    # along +z from the origin: segment z in [0.3, 0.5], cells of 0.08 -> z cells 3, 4, 5, 6
    keys = O.collect_band_blocks(np.full((1, 1), 0.4, np.float32), K, eye, 0.01, 0.1)
    assert keys.tolist() == [[0, 0, 3], [0, 0, 4], [0, 0, 5], [0, 0, 6]]
    # no valid depth, no keys
    assert O.collect_band_blocks(np.zeros((1, 1), np.float32), K, eye, 0.01, 0.1).shape == (0, 3)
    # a camera far outside the 21-bit key range: overflow is reported, as for the reference rule
    far = scenes.Pose(np.eye(3, dtype=np.float32), np.array([1.0e6, 0.0, 0.0], np.float32))
    assert O.collect_band_blocks(np.full((1, 1), 0.4, np.float32), K, far, 0.01, 0.1) is None


def test_band_rule_is_a_walk_of_the_segment(O):
    """On a rendered frame: the band holds the cells that dense samples of each segment fall in (those clear of a
    cell face), and the band lies inside the reference rule's 3 x 27 neighbourhood (a segment of half-length
    trunc < 8 vs stays within one cell of p)."""
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=5, frames=4, width=40, height=30, fx=36.0, fy=36.0, cx=19.5, cy=14.5)
    K = sc.intrinsics
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN)
    bws = 8 * sc.voxel_size
    for f in (0, 2):
        d = scenes.render_depth(sc, f)
        band = O.collect_band_blocks(d, K, sc.poses[f], sc.voxel_size, sc.truncation)
        ref = O.collect_blocks(cfg, d, K, sc.poses[f], sc.voxel_size, sc.truncation)
        band_set = {tuple(k) for k in band}
        assert len(band_set) == band.shape[0] and band_set <= {tuple(k) for k in ref}
        assert len(band_set) < ref.shape[0]
        v, u = np.nonzero(d > 0)
        z = d[v, u].astype(np.float64)
        pc = np.stack([(u - K.cx) * z / K.fx, (v - K.cy) * z / K.fy, z], 1)
        R = np.asarray(sc.poses[f].R, np.float64)
        t = np.asarray(sc.poses[f].t, np.float64)
        pw = pc @ R.T + t
        ray = (pw - t) / np.linalg.norm(pw - t, axis=1, keepdims=True)
        for s in np.linspace(-1.0, 1.0, 65):
            g = (pw + ray * (s * sc.truncation)) / bws
            frac = g - np.floor(g)
            safe = np.all((frac > 1e-3) & (frac < 1 - 1e-3), axis=1)
            need = {tuple(k) for k in np.floor(g[safe]).astype(np.int64).tolist()}
            assert need <= band_set, "a cell on a pixel's segment is missing from the band"


def test_fp64_transcription_bounds_the_float_path(O):
    """The restatement (float arithmetic, bit-identical to the reference and to the product's plain form) against
    the same equations in FP64 (oracle/liboracle64.so), on the small orbit scene over four frames.  Stated
    tolerances: filtered depth within 1e-6 relative with the same valid pixels; the same block keys; per layer
    occupied in both, weight and surface coordinate within 1e-5 relative to max(|x|, 1) for all but 1e-4 of
    the layers (the rest are observations that a rounding moved to another layer), plane offset within 1e-5 at
    the 99th percentile; marching-cubes vertices within 1e-4 voxel at the median and 1e-2 voxel at the 99th
    percentile (interpolation divides by corner-value differences)."""
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=7, frames=24, width=64, height=48, fx=277.0 * 0.2, fy=277.0 * 0.2, cx=32.0, cy=24.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    K = sc.intrinsics
    cfg = O.config(O.FLAVOR_REF_GPU, O.EXP_OWN, threads=4)
    v32 = O.Volume(cfg, sc.voxel_size, sc.truncation)
    v64 = O.Volume(cfg, sc.voxel_size, sc.truncation, fp64=True)
    for f in (0, 6, 12, 18):
        d = scenes.render_depth(sc, f)
        a, b = O.filter_depth(cfg, d, K), O.filter_depth(cfg, d, K, fp64=True)
        assert np.array_equal(a > 0, b > 0)
        ok = b > 0
        assert np.max(np.abs(a[ok].astype(np.float64) - b[ok]) / b[ok]) <= 1e-6
        k32 = O.collect_blocks(cfg, d, K, sc.poses[f], sc.voxel_size, sc.truncation)
        k64 = O.collect_blocks(cfg, d, K, sc.poses[f], sc.voxel_size, sc.truncation, fp64=True)
        assert np.array_equal(k32, k64)
        v32.integrate(d, K, sc.poses[f], 1)
        v64.integrate(d, K, sc.poses[f], 1)
    ka, xa = O.sort_blocks(*v32.blocks())
    kb, xb = O.sort_blocks(*v64.blocks())
    assert np.array_equal(ka, kb)
    occ_a, occ_b = xa["weight"] > 0, xb["weight"] > 0
    both = occ_a & occ_b
    assert (occ_a != occ_b).sum() <= 1e-4 * both.sum()
    rel = {}
    for name in ("weight", "surface_coord", "plane_offset"):
        x, y = xa[name][both].astype(np.float64), xb[name][both].astype(np.float64)
        rel[name] = np.abs(x - y) / np.maximum(np.abs(y), 1.0)
    assert (rel["weight"] > 1e-5).mean() <= 1e-4
    assert (rel["surface_coord"] > 1e-5).mean() <= 1e-4
    assert np.quantile(rel["plane_offset"], 0.99) <= 1e-5
    from scipy.spatial import cKDTree
    ta, tb = v32.extract_mesh(), v64.extract_mesh()
    assert abs(ta.shape[0] - tb.shape[0]) <= 1e-3 * tb.shape[0]
    dist = cKDTree(tb.reshape(-1, 3).astype(np.float64)).query(ta.reshape(-1, 3).astype(np.float64))[0]
    dist /= sc.voxel_size
    assert np.median(dist) <= 1e-4 and np.quantile(dist, 0.99) <= 1e-2
    assert v32.observed_voxels() == v64.observed_voxels()


@pytest.mark.parametrize("kind", ["orbit", "room", "object_scan"])
def test_renderer_restatement_matches_float64_render(O, kind):
    """The host restatement of the device renderer (FP32 geometry, own FP64 noise functions) against the
    float64 numpy renderer of voxelhashmt_gb300/scenes.py: the same valid pixels and dropouts, depth within
    2e-4 relative (FP32 ray geometry at grazing angles) and 2e-5 at the 99.9th percentile; noise-free frames
    the same."""
    from voxelhashmt_gb300 import scenes
    sc = {"orbit": lambda: scenes.orbit_scene(seed=3, frames=8),
          "room": lambda: scenes.room_scene(seed=1, frames=4),
          "object_scan": lambda: scenes.object_scan_scene(seed=5)}[kind]()
    for frame in (0, 1):
        for noise in (True, False):
            a = O.render_depth(sc, frame, noise=noise)
            b = scenes.render_depth(sc, frame, noise=noise)
            assert np.array_equal(a > 0, b > 0)
            both = (a > 0) & (b > 0)
            assert both.sum() > 1000
            rel = np.abs(a[both].astype(np.float64) - b[both]) / b[both]
            assert rel.max() <= 2e-4 and np.quantile(rel, 0.999) <= 2e-5, (float(rel.max()), frame, noise)


def test_reciprocal_root_is_correctly_rounded(O):
    """The oracle's restatement of the FP16 codec's normalisation (the device's __frsqrt_rn, correctly rounded
    by definition) returns the float nearest to 1/sqrt(x), checked at 100 digits on the squared lengths of
    octahedral directions, [1/3, 1]: a seeded sample and both ends."""
    import ctypes as C
    import mpmath
    L = O.lib()
    L.vo_rsqrtf_rn.argtypes = [C.c_float]
    L.vo_rsqrtf_rn.restype = C.c_float
    mpmath.mp.dps = 100
    rng = np.random.default_rng(8)
    lo, hi = int(np.float32(1.0 / 3.0).view(np.uint32)), int(np.float32(1.0).view(np.uint32))
    bits = np.concatenate([rng.integers(lo, hi + 1, 20000), np.arange(lo, lo + 50), np.arange(hi - 50, hi + 1)])
    for b in bits.astype(np.uint32):
        x = float(np.uint32(b).view(np.float32))
        got = np.float32(L.vo_rsqrtf_rn(x))
        exact = 1 / mpmath.sqrt(mpmath.mpf(x))
        up, dn = np.nextafter(got, np.float32(2)), np.nextafter(got, np.float32(0))
        err = abs(mpmath.mpf(float(got)) - exact)
        assert err <= abs(mpmath.mpf(float(up)) - exact) and err <= abs(mpmath.mpf(float(dn)) - exact), x
