"""CPU tests of the dataset reader (voxelhashmt_gb300/csrc/vh_dataset.cpp, vh_png.cpp; the reference's
include/tsdfmc/dataset_io.h).

* PNG decoding against files written here with Python's zlib (stored, fixed and dynamic DEFLATE blocks):
  grayscale bit depths 1-16, gray + alpha, all five scanline filters, Adam7 interlacing; corrupt files and
  colour images are refused with a message.
* Dataset layout: frame-id listing, pose files (quaternion, 3x4, 4x4), intrinsics metadata (5, 6, 7 values,
  params.txt fallback, resolution from the first depth.png), depth scaling and validity counting.
* Against the reference's own dataset_io.h compiled here (where the reference tree is present): poses,
  intrinsics and frame ids are bit-identical.
"""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def ds(product_lib):
    from voxelhashmt_gb300 import dataset
    return dataset


def _chunk(kind, body):
    c = kind + body
    return struct.pack(">I", len(body)) + c + struct.pack(">I", zlib.crc32(c) & 0xffffffff)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_rows(raw_rows, bpp, filters):
    """raw_rows: list of uint8 arrays (one scanline each); returns the filtered stream with type bytes."""
    out = bytearray()
    prev = np.zeros_like(raw_rows[0]) if raw_rows else None
    for y, row in enumerate(raw_rows):
        ft = filters[y % len(filters)]
        r = row.astype(np.int32)
        p = prev.astype(np.int32)
        a = np.concatenate([np.zeros(bpp, np.int32), r[:-bpp]]) if len(r) > bpp else np.zeros_like(r)
        c = np.concatenate([np.zeros(bpp, np.int32), p[:-bpp]]) if len(p) > bpp else np.zeros_like(p)
        if len(r) <= bpp:
            a = np.zeros_like(r)
            c = np.zeros_like(r)
        pred = [np.zeros_like(r), a, p, (a + p) >> 1, _paeth(a, p, c)][ft]
        out.append(ft)
        out += ((r - pred) & 0xff).astype(np.uint8).tobytes()
        prev = row
    return bytes(out)


def _pack_rows(img, depth, channels):
    """(H, W[, C]) integer samples -> list of packed scanlines."""
    h, w = img.shape[:2]
    samples = img.reshape(h, w * channels).astype(np.uint32)
    rows = []
    for y in range(h):
        s = samples[y]
        if depth == 16:
            rows.append(np.stack([(s >> 8) & 0xff, s & 0xff], 1).reshape(-1).astype(np.uint8))
        elif depth == 8:
            rows.append(s.astype(np.uint8))
        else:
            per = 8 // depth
            pad = (-len(s)) % per
            s2 = np.concatenate([s, np.zeros(pad, np.uint32)]).reshape(-1, per)
            shifts = np.array([8 - depth * (k + 1) for k in range(per)], np.uint32)
            rows.append((s2 << shifts).sum(1).astype(np.uint8))
    return rows


ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def write_png(path, img, depth, ctype=0, filters=(0, 1, 2, 3, 4), level=6, interlace=False, corrupt_crc=False):
    channels = {0: 1, 4: 2, 2: 3}[ctype]
    h, w = img.shape[:2]
    bits = depth * channels
    bpp = max(1, bits // 8)
    if interlace:
        stream = b""
        for x0, y0, dx, dy in ADAM7:
            sub = img[y0::dy, x0::dx]
            if sub.shape[0] == 0 or sub.shape[1] == 0:
                continue
            stream += _filter_rows(_pack_rows(sub, depth, channels), bpp, filters)
    else:
        stream = _filter_rows(_pack_rows(img, depth, channels), bpp, filters)
    ihdr = struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0)
    data = zlib.compress(stream, level)
    idat = _chunk(b"IDAT", data[: len(data) // 2]) + _chunk(b"IDAT", data[len(data) // 2:])  # split across chunks
    if corrupt_crc:
        idat = idat[:-1] + bytes([idat[-1] ^ 1])
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"tEXt", b"k\x00v") + idat + _chunk(b"IEND", b""))


@pytest.mark.parametrize("depth", [1, 2, 4, 8, 16])
@pytest.mark.parametrize("interlace", [False, True])
def test_png_grayscale_depths(ds, tmp_path, depth, interlace):
    rng = np.random.default_rng(depth * 10 + interlace)
    img = rng.integers(0, 1 << depth, size=(37, 29), dtype=np.uint32)
    for level in (0, 1, 9):
        p = tmp_path / ("g%d_%d_%d.png" % (depth, interlace, level))
        write_png(p, img, depth, interlace=interlace, level=level)
        got = ds.read_depth_png_gray16(p)
        want = (img * 65535 // ((1 << depth) - 1)).astype(np.uint16)
        assert got.shape == img.shape and np.array_equal(got, want)


@pytest.mark.parametrize("depth", [8, 16])
def test_png_gray_alpha_and_smooth_depth(ds, tmp_path, depth):
    rng = np.random.default_rng(depth)
    yy, xx = np.mgrid[0:48, 0:64]
    gray = ((1500 + 3 * xx + 7 * yy) % (1 << depth)).astype(np.uint32)  # smooth: long DEFLATE matches
    alpha = rng.integers(0, 1 << depth, size=gray.shape, dtype=np.uint32)
    p = tmp_path / "ga.png"
    write_png(p, np.stack([gray, alpha], -1), depth, ctype=4, filters=(4, 3, 2, 1, 0))
    got = ds.read_depth_png_gray16(p)
    assert np.array_equal(got, (gray * (65535 // ((1 << depth) - 1))).astype(np.uint16))


def test_png_refuses_bad_input(ds, tmp_path):
    img = np.arange(20, dtype=np.uint32).reshape(4, 5)
    bad = tmp_path / "bad.png"
    write_png(bad, img, 16, corrupt_crc=True)
    with pytest.raises(RuntimeError, match="CRC"):
        ds.read_depth_png_gray16(bad)
    rgb = tmp_path / "rgb.png"
    write_png(rgb, np.stack([img, img, img], -1), 8, ctype=2)
    with pytest.raises(RuntimeError, match="grayscale"):
        ds.read_depth_png_gray16(rgb)
    trunc = tmp_path / "trunc.png"
    good = tmp_path / "good.png"
    write_png(good, img, 16)
    trunc.write_bytes(good.read_bytes()[:40])
    with pytest.raises(RuntimeError):
        ds.read_depth_png_gray16(trunc)
    with pytest.raises(RuntimeError, match="open"):
        ds.read_depth_png_gray16(tmp_path / "missing.png")


def _write_numbers(path, values):
    path.write_text(" ".join(repr(float(v)) for v in values) + "\n")


def make_dataset(root, scene, frames, depth_scale=0.001, pose_kind="quat"):
    """A dataset of `frames` of an analytic scene: depth quantised to depth_scale, poses from the scene."""
    from scipy.spatial.transform import Rotation
    from voxelhashmt_gb300 import scenes
    os.makedirs(root / "notaframe", exist_ok=True)
    for f in frames:
        d = root / str(f)
        d.mkdir(parents=True, exist_ok=True)
        depth = scenes.render_depth(scene, f)
        raw = np.round(depth / depth_scale).astype(np.uint32)
        write_png(d / "depth.png", np.minimum(raw, 65535), 16, filters=(1, 2, 4))
        P = scene.poses[f]
        R = np.asarray(P.R, np.float64)
        t = np.asarray(P.t, np.float64)
        if pose_kind == "quat":
            x, y, z, w = Rotation.from_matrix(R).as_quat()
            _write_numbers(d / "pose.txt", [w, x, y, z, *t])
        else:
            M = np.eye(4)
            M[:3, :3], M[:3, 3] = R, t
            _write_numbers(d / "pose.txt", M.reshape(-1)[:12] if pose_kind == "3x4" else M.reshape(-1))
    return root


def test_dataset_layout_round_trip(ds, tmp_path):
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=2, frames=12, width=48, height=36, fx=41.5, fy=41.5, cx=24.0, cy=18.0)
    root = make_dataset(tmp_path / "ds", sc, [10, 2, 0], pose_kind="quat")
    assert ds.list_dataset_frame_ids(root) == [0, 2, 10]
    # 5 values: resolution from the first depth.png
    _write_numbers(root / "intrinsics.txt", [41.5, 41.5, 24.0, 18.0, 0.001])
    K, scale = ds.load_dataset_intrinsics(root / "intrinsics.txt")
    assert (K.width, K.height, K.fx, K.cy) == (48, 36, 41.5, 18.0) and scale == np.float32(0.001)
    # missing file: falls back to the first <frame>/params.txt (7 values)
    _write_numbers(root / "2" / "params.txt", [41.5, 41.5, 24.0, 18.0, 48, 36, 0.001])
    K2, s2 = ds.load_dataset_intrinsics(root / "absent.txt")
    assert (K2.width, K2.height) == (48, 36) and s2 == np.float32(0.001)
    for f in (0, 2, 10):
        fr = ds.load_dataset_depth_frame(root, f, "pose.txt", K, scale)
        want = np.round(scenes.render_depth(sc, f) / 0.001).astype(np.uint32)
        want_depth = np.where(want > 0, want.astype(np.float32) * np.float32(0.001), 0).astype(np.float32)
        assert np.array_equal(fr.depth_frame.depth, want_depth)
        assert fr.valid_depth_samples == int(np.count_nonzero(want))
        assert np.allclose(fr.T_wc.R, sc.poses[f].R, atol=1e-6) and np.allclose(fr.T_wc.t, sc.poses[f].t, atol=1e-6)
    for kind in ("3x4", "4x4"):
        r2 = make_dataset(tmp_path / kind, sc, [3], pose_kind=kind)
        P = ds.load_pose_from_file(r2 / "3" / "pose.txt")
        assert np.array_equal(P.R, np.asarray(sc.poses[3].R, np.float32))
    # errors carry the reference's messages
    bad = tmp_path / "bad_pose.txt"
    _write_numbers(bad, [1, 2, 3])
    with pytest.raises(RuntimeError, match="Unsupported pose format"):
        ds.load_pose_from_file(bad)
    wrong = type(K)(K.width + 1, K.height, K.fx, K.fy, K.cx, K.cy)
    with pytest.raises(RuntimeError, match="resolution does not match"):
        ds.load_depth_png(root / "0" / "depth.png", wrong, scale)


def _reference_present():
    from oracle import build as ob
    return ob.reference_available()


ref_only = pytest.mark.skipif(not _reference_present(), reason="reference tree not present on this machine")


@ref_only
def test_dataset_matches_reference_reader(ds, tmp_path):
    """Poses, intrinsics (6- and 7-value files) and frame ids against dataset_io.h compiled here."""
    from oracle import build as ob
    exe = ob.build_ref_dataset()
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=4, frames=8, width=32, height=24, fx=27.7, fy=27.7, cx=16.0, cy=12.0)
    root = make_dataset(tmp_path / "ds", sc, [7, 1, 4], pose_kind="quat")
    rng = np.random.default_rng(0)
    files = []
    for i in range(20):  # random quaternions (unnormalised) and matrices
        p = tmp_path / ("q%d.txt" % i)
        _write_numbers(p, list(rng.normal(size=4) * rng.uniform(0.1, 10)) + list(rng.normal(size=3)))
        files.append(p)
        m = tmp_path / ("m%d.txt" % i)
        _write_numbers(m, rng.normal(size=16 if i % 2 else 12))
        files.append(m)
    files.append(root / "1" / "pose.txt")
    for p in files:
        ref = subprocess.run([exe, "pose", str(p)], capture_output=True, text=True, check=True).stdout.split()
        P = ds.load_pose_from_file(p)
        ours = np.concatenate([np.asarray(P.R, np.float32).reshape(-1), np.asarray(P.t, np.float32)])
        assert [int(x, 16) for x in ref] == [int(v) for v in ours.view(np.uint32)], p
    for vals in ([525.0, 525.0, 319.5, 239.5, 640, 480], [277.1, 276.9, 160.25, 119.75, 320, 240, 0.0002]):
        p = tmp_path / "intr.txt"
        _write_numbers(p, vals)
        ref = subprocess.run([exe, "intrinsics", str(p)], capture_output=True, text=True, check=True).stdout.split()
        K, scale = ds.load_dataset_intrinsics(p)
        ours = [K.width, K.height] + [int(v) for v in np.array([K.fx, K.fy, K.cx, K.cy, scale], np.float32).view(np.uint32)]
        assert [int(ref[0]), int(ref[1])] + [int(x, 16) for x in ref[2:]] == ours
    ref = subprocess.run([exe, "frames", str(root)], capture_output=True, text=True, check=True).stdout.split()
    assert [int(x) for x in ref] == ds.list_dataset_frame_ids(root)
