"""Mesh output: the reference's PLY triangle soup and an indexed (welded) mesh.

* ``write_ply_soup`` writes the file the reference's writeMeshAsPly writes (src/main.cpp:337-398): binary
  little-endian PLY, triangles with norm(cross(v1 - v0, v2 - v0)) <= 1e-8 dropped, three unshared vertices per
  face, each carrying the face's unit normal, face list `uchar 3, int i, i+1, i+2`.  All arithmetic is float32
  in the reference's order, so the bytes match apart from the comment line.
* ``weld`` turns the soup from extract_mesh into an indexed mesh.  Vertices are merged only when their three
  float32 coordinates are bit-identical.  Neighbouring marching-cubes cells recompute a shared edge's vertex
  from their own cluster centres, so only bit-identical copies are the same point.  Vertices are numbered by
  first use and faces keep the soup's order, so the device weld (vh_weld_mesh, backend.extract_mesh_indexed)
  returns the same arrays.
* ``write_ply_indexed`` writes the welded mesh with area-weighted vertex normals.
"""
from __future__ import annotations

import numpy as np

_FACE_DTYPE = np.dtype([("n", "u1"), ("i", "<i4", (3,))])


def _cross(a, b):
    """math_types.h:83-89 in float32."""
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1).astype(np.float32)


def _norm(v):
    """sqrt(dot(v, v)) with dot = (x*x + y*y) + z*z, float32."""
    return np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]).astype(np.float32)


def _normalized(v):
    """math_types.h:95-101: v / |v|, zero when |v| <= 1e-8."""
    n = _norm(v)
    out = np.zeros_like(v)
    ok = n > np.float32(1e-8)
    out[ok] = v[ok] / n[ok, None]
    return out


def face_normals(tris):
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    return _cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])


def write_ply_soup(path, tris, comment="generated by voxelhashmt_gb300"):
    """The reference's writeMeshAsPly (src/main.cpp:337-398) for an (N, 9) float32 triangle soup."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    cr = face_normals(t)
    keep = _norm(cr) > np.float32(1e-8)
    t, cr = t[keep], cr[keep]
    unit = _normalized(cr)
    f = t.shape[0]
    vert = np.concatenate([t, np.repeat(unit[:, None, :], 3, axis=1)], axis=2).reshape(-1, 6).astype("<f4")
    faces = np.zeros(f, _FACE_DTYPE)
    faces["n"] = 3
    faces["i"] = np.arange(3 * f, dtype=np.int32).reshape(f, 3)
    header = ("ply\nformat binary_little_endian 1.0\ncomment %s\nelement vertex %d\nproperty float x\n"
              "property float y\nproperty float z\nproperty float nx\nproperty float ny\nproperty float nz\n"
              "element face %d\nproperty list uchar int vertex_indices\nend_header\n" % (comment, 3 * f, f))
    with open(path, "wb") as fh:
        fh.write(header.encode("ascii"))
        fh.write(vert.tobytes())
        fh.write(faces.tobytes())
    return f


def weld(tris):
    """(vertices (V, 3) float32, faces (F, 3) int32) from a soup; vertices merged when bit-identical and numbered
    in the order of their first use in the soup; faces keep the soup's order, and faces that collapse (a
    repeated index) or have zero area are dropped.  The device weld (vh_weld_mesh) gives the same arrays."""
    t = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 3))
    if t.shape[0] == 0:
        return np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)
    keys = t.view(np.uint32)
    _, first, inverse = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")  # unique keys by first use
    rank = np.empty(order.shape[0], np.int64)
    rank[order] = np.arange(order.shape[0])
    verts = t[first[order]]
    faces = rank[inverse.reshape(-1)].reshape(-1, 3).astype(np.int32)
    ok = (faces[:, 0] != faces[:, 1]) & (faces[:, 1] != faces[:, 2]) & (faces[:, 0] != faces[:, 2])
    faces = faces[ok]
    area = _norm(_cross(verts[faces[:, 1]] - verts[faces[:, 0]], verts[faces[:, 2]] - verts[faces[:, 0]]))
    return verts, faces[area > np.float32(1e-8)]


def vertex_normals(verts, faces):
    n = np.zeros_like(verts, dtype=np.float64)
    fn = _cross(verts[faces[:, 1]] - verts[faces[:, 0]], verts[faces[:, 2]] - verts[faces[:, 0]]).astype(np.float64)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    length = np.linalg.norm(n, axis=1, keepdims=True)
    return (n / np.maximum(length, 1e-30)).astype(np.float32)


def write_ply_indexed(path, verts, faces, comment="generated by voxelhashmt_gb300 (welded)"):
    verts = np.asarray(verts, np.float32)
    faces = np.asarray(faces, np.int32)
    vert = np.concatenate([verts, vertex_normals(verts, faces)], axis=1).astype("<f4")
    fr = np.zeros(faces.shape[0], _FACE_DTYPE)
    fr["n"] = 3
    fr["i"] = faces
    header = ("ply\nformat binary_little_endian 1.0\ncomment %s\nelement vertex %d\nproperty float x\n"
              "property float y\nproperty float z\nproperty float nx\nproperty float ny\nproperty float nz\n"
              "element face %d\nproperty list uchar int vertex_indices\nend_header\n"
              % (comment, verts.shape[0], faces.shape[0]))
    with open(path, "wb") as fh:
        fh.write(header.encode("ascii"))
        fh.write(vert.tobytes())
        fh.write(fr.tobytes())


def read_ply(path):
    """(vertices (V, 6) float32 [x y z nx ny nz], faces (F, 3) int32) of a file written by either writer (or by
    the reference)."""
    with open(path, "rb") as fh:
        data = fh.read()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    header = data[:end].decode("ascii").splitlines()
    nv = int(next(h for h in header if h.startswith("element vertex")).split()[-1])
    nf = int(next(h for h in header if h.startswith("element face")).split()[-1])
    vert = np.frombuffer(data, "<f4", count=nv * 6, offset=end).reshape(nv, 6)
    faces = np.frombuffer(data, _FACE_DTYPE, count=nf, offset=end + nv * 24)
    return vert.copy(), faces["i"].copy()
