"""Reconstruction quality against the analytic scene: Chamfer distance of a fused mesh.

* accuracy: mean distance from the mesh vertices to the analytic surface (exact distance to the union of the
  scene's primitives, scenes.scene_sdf);
* completeness: mean distance from points of the observed surface to the mesh (exact point-triangle
  distance).  The points come from noise-free renders of frames that were fused, so they lie on the
  analytic surface and only in regions the camera saw.
* chamfer = (accuracy + completeness) / 2.

All distances in millimetres.
"""
from __future__ import annotations

import numpy as np

from . import scenes


def observed_surface_points(scene, frames, depth_maps=None, stride=4, max_points=200_000, seed=0):
    """World points of noise-free depth pixels of `frames` (every `stride`-th pixel), subsampled to
    max_points.  depth_maps: optional noise-free depth per frame (e.g. from the device renderer)."""
    K = scene.intrinsics
    pts = []
    for n, f in enumerate(frames):
        d = depth_maps[n] if depth_maps is not None else scenes.render_depth(scene, f, noise=False)
        d = np.asarray(d, np.float64)[::stride, ::stride]
        v, u = np.nonzero(d > 0)
        z = d[v, u]
        uu, vv = u * stride, v * stride
        pc = np.stack([(uu - K.cx) * z / K.fx, (vv - K.cy) * z / K.fy, z], axis=1)
        P = scene.poses[f]
        pts.append(pc @ np.asarray(P.R, np.float64).T + np.asarray(P.t, np.float64))
    pts = np.concatenate(pts) if pts else np.zeros((0, 3))
    if pts.shape[0] > max_points:
        pts = pts[np.random.default_rng(seed).choice(pts.shape[0], max_points, replace=False)]
    return pts


def point_triangle_distance(p, a, b, c):
    """Euclidean distance from points p (N, 3) to triangles (a, b, c) (N, 3 each), float64: the closest point
    by Voronoi-region tests on the triangle (Ericson, Real-Time Collision Detection, 2005, sec. 5.1.5);
    degenerate triangles fall back to the nearest vertex or edge point."""
    p, a, b, c = (np.asarray(x, np.float64) for x in (p, a, b, c))
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = np.einsum("ij,ij->i", ab, ap), np.einsum("ij,ij->i", ac, ap)
    bp = p - b
    d3, d4 = np.einsum("ij,ij->i", ab, bp), np.einsum("ij,ij->i", ac, bp)
    cp = p - c
    d5, d6 = np.einsum("ij,ij->i", ab, cp), np.einsum("ij,ij->i", ac, cp)
    va = d3 * d6 - d5 * d4
    vb = d5 * d2 - d1 * d6
    vc = d1 * d4 - d3 * d2
    q = np.empty_like(p)
    done = np.zeros(p.shape[0], bool)

    def put(mask, val):
        m = mask & ~done
        q[m] = val[m] if val.ndim == 2 else val
        done[:] |= m

    eps = 1e-300
    put((d1 <= 0) & (d2 <= 0), a)
    put((d3 >= 0) & (d4 <= d3), b)
    v = d1 / np.where(np.abs(d1 - d3) > eps, d1 - d3, eps)
    put((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + v[:, None] * ab)
    put((d6 >= 0) & (d5 <= d6), c)
    w = d2 / np.where(np.abs(d2 - d6) > eps, d2 - d6, eps)
    put((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + w[:, None] * ac)
    den = (d4 - d3) + (d5 - d6)
    w = (d4 - d3) / np.where(np.abs(den) > eps, den, eps)
    put((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0), b + w[:, None] * (c - b))
    s = va + vb + vc
    s = np.where(np.abs(s) > eps, s, eps)
    put(np.ones(p.shape[0], bool), a + (vb / s)[:, None] * ab + (vc / s)[:, None] * ac)
    return np.linalg.norm(p - q, axis=1)


def chamfer(tris, scene, surface_points, max_accuracy_triangles=1_000_000, neighbours=8, seed=0):
    """Accuracy, completeness and Chamfer distance (mm) of a triangle soup against the analytic scene.

    accuracy: mean |scene SDF| over the vertices of (up to max_accuracy_triangles seeded) triangles;
    completeness: mean distance from the surface points to the mesh, the exact point-triangle distance
    minimised over the `neighbours` triangles with the nearest centroids."""
    from scipy.spatial import cKDTree
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    if t.shape[0] == 0:
        inf = float("inf")
        return {"accuracy_mm": inf, "completeness_mm": inf, "chamfer_mm": inf, "accuracy_p90_mm": inf,
                "triangles": 0}
    rng = np.random.default_rng(seed)
    ta = t if t.shape[0] <= max_accuracy_triangles else t[rng.choice(t.shape[0], max_accuracy_triangles,
                                                                    replace=False)]
    acc = np.abs(scenes.scene_sdf(scene.prims, ta.reshape(-1, 3).astype(np.float64)))
    cent = t.mean(axis=1)
    tree = cKDTree(cent, balanced_tree=False, compact_nodes=False)
    sp = np.asarray(surface_points, np.float64)
    k = min(neighbours, t.shape[0])
    _, idx = tree.query(sp, k=k)
    idx = idx.reshape(sp.shape[0], k)
    best = np.full(sp.shape[0], np.inf)
    for j in range(k):
        tj = t[idx[:, j]].astype(np.float64)
        best = np.minimum(best, point_triangle_distance(sp, tj[:, 0], tj[:, 1], tj[:, 2]))
    a, c = 1000.0 * float(np.mean(acc)), 1000.0 * float(np.mean(best))
    return {"accuracy_mm": a, "completeness_mm": c, "chamfer_mm": 0.5 * (a + c),
            "accuracy_p90_mm": 1000.0 * float(np.quantile(acc, 0.9)),
            "completeness_p90_mm": 1000.0 * float(np.quantile(best, 0.9)), "triangles": int(t.shape[0])}
