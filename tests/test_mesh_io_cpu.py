"""Mesh output: the reference's PLY soup format (byte-compatible) and the welded indexed mesh."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def soup(oracle_lib):
    from voxelhashmt_gb300 import scenes
    O = oracle_lib
    sc = scenes.orbit_scene(seed=9, frames=6, width=40, height=30, fx=34.6, fy=34.6, cx=20.0, cy=15.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    v = O.Volume(O.config(O.FLAVOR_REF_GPU, O.EXP_OWN, threads=4), sc.voxel_size, sc.truncation)
    for f in (0, 2):
        v.integrate(scenes.render_depth(sc, f), sc.intrinsics, sc.poses[f])
    t = v.extract_mesh()
    v.close()
    assert t.shape[0] > 100
    return t


def test_soup_round_trip(soup, tmp_path):
    from voxelhashmt_gb300 import mesh_io
    path = os.path.join(ROOT, "oracle", "_ref") if os.path.isdir(os.path.join(ROOT, "oracle", "_ref")) else tmp_path
    out = os.path.join(str(path), "soup_roundtrip.ply")
    f = mesh_io.write_ply_soup(out, soup)
    vert, faces = mesh_io.read_ply(out)
    keep = np.sqrt(np.sum(mesh_io.face_normals(soup).astype(np.float64) ** 2, axis=1)) > 1e-8
    assert f == int(keep.sum()) == faces.shape[0] and vert.shape[0] == 3 * f
    assert np.array_equal(vert[:, :3].reshape(-1, 9).view(np.uint32), soup[keep].view(np.uint32))
    assert np.array_equal(faces, np.arange(3 * f, dtype=np.int32).reshape(f, 3))
    os.remove(out)


def test_weld_merges_only_bit_identical_vertices(soup):
    from voxelhashmt_gb300 import mesh_io
    verts, faces = mesh_io.weld(soup)
    pts = soup.reshape(-1, 3)
    assert verts.shape[0] == np.unique(pts.view(np.uint32), axis=0).shape[0] < pts.shape[0]
    # every kept face reproduces a soup triangle exactly
    got = verts[faces].reshape(-1, 9)
    soup_set = {row.tobytes() for row in soup.view(np.uint32)}
    assert all(row.tobytes() in soup_set for row in got.view(np.uint32))
    assert faces.shape[0] <= soup.shape[0]


def test_soup_writer_matches_reference_writer_bytes(reference_demo):
    """The reference demo (CPU backend) writes its mesh with writeMeshAsPly; re-writing its triangles with
    write_ply_soup reproduces the file byte for byte apart from the comment line."""
    from voxelhashmt_gb300 import mesh_io
    out = os.path.join(ROOT, "oracle", "_ref", "ref_demo_cpu.ply")
    res = subprocess.run([reference_demo, "--synthetic", "--backend", "cpu", "--frames", "2", "--width", "40",
                          "--height", "30", "--voxel-size", "0.02", "--truncation", "0.06", "--output", out],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    vert, faces = mesh_io.read_ply(out)
    assert faces.shape[0] > 0
    tris = vert[:, :3].reshape(-1, 9)
    mine = out + ".gb300.ply"
    mesh_io.write_ply_soup(mine, tris, comment="generated by tsdf_voxel_hash_demo")
    assert open(out, "rb").read() == open(mine, "rb").read()
    os.remove(mine)


def test_weld_known_answer():
    """Vertices numbered by first use, faces in soup order; a collapsed face and a zero-area face dropped; -0.0
    and 0.0 are different bit patterns and stay different vertices."""
    from voxelhashmt_gb300 import mesh_io
    A, B, C, D = [0.0, 0.0, 1.0], [1.0, 0.0, 1.0], [0.0, 1.0, 1.0], [1.0, 1.0, 1.0]
    E, F, G = [2.0, 0.0, 0.0], [3.0, 0.0, 0.0], [4.0, 0.0, 0.0]  # collinear
    Z, Zm = [0.0, 0.0, 0.0], [-0.0, 0.0, 0.0]
    soup = np.array([A + B + C, C + B + D, A + A + B, E + F + G, D + C + E, Z + A + B, Zm + C + D], np.float32)
    verts, faces = mesh_io.weld(soup)
    want_v = np.array([A, B, C, D, E, F, G, Z, Zm], np.float32)
    assert np.array_equal(verts.view(np.uint32), want_v.view(np.uint32))
    assert faces.tolist() == [[0, 1, 2], [2, 1, 3], [3, 2, 4], [7, 0, 1], [8, 2, 3]]
    v0, f0 = mesh_io.weld(np.zeros((0, 9), np.float32))
    assert v0.shape == (0, 3) and f0.shape == (0, 3)


def test_indexed_ply_round_trip(soup, tmp_path):
    """The welded mesh written as an indexed PLY reads back with the same vertices and faces, and unit
    area-weighted vertex normals."""
    from voxelhashmt_gb300 import mesh_io
    verts, faces = mesh_io.weld(soup)
    out = os.path.join(str(tmp_path), "welded.ply")
    mesh_io.write_ply_indexed(out, verts, faces)
    v, f = mesh_io.read_ply(out)
    assert np.array_equal(v[:, :3].view(np.uint32), verts.view(np.uint32))
    assert np.array_equal(f, faces)
    length = np.linalg.norm(v[:, 3:].astype(np.float64), axis=1)
    used = np.zeros(verts.shape[0], bool)
    used[faces.reshape(-1)] = True
    assert np.allclose(length[used], 1.0, atol=1e-5)
