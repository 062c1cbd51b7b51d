"""CPU tests of the reconstruction-quality metric (voxelhashmt_gb300/metrics.py)."""
import numpy as np


def test_point_triangle_distance_against_dense_sampling():
    from voxelhashmt_gb300 import metrics
    rng = np.random.default_rng(0)
    n = 3000
    a, b, c = rng.normal(size=(3, n, 3))
    p = rng.normal(size=(n, 3)) * 2
    d = metrics.point_triangle_distance(p, a, b, c)
    m = 120
    best = np.full(n, np.inf)
    for i in range(m + 1):
        for j in range(m + 1 - i):
            q = a + (i / m) * (b - a) + (j / m) * (c - a)
            best = np.minimum(best, np.linalg.norm(p - q, axis=1))
    # exact distance <= any sampled point's, and within the sampling spacing of the best sample
    edge = np.maximum(np.linalg.norm(b - a, axis=1), np.linalg.norm(c - a, axis=1))
    assert np.all(d <= best + 1e-12)
    assert np.all(best - d <= edge / m + 1e-9)


def test_point_triangle_distance_regions():
    from voxelhashmt_gb300 import metrics
    a, b, c = np.array([[0.0, 0, 0]]), np.array([[1.0, 0, 0]]), np.array([[0.0, 1, 0]])
    cases = {(0.2, 0.2, 0.5): 0.5, (-1.0, -1.0, 0.0): np.sqrt(2.0), (0.5, -2.0, 0.0): 2.0,
             (1.0, 1.0, 0.0): np.sqrt(0.5), (3.0, 0.0, 0.0): 2.0}
    for p, want in cases.items():
        got = metrics.point_triangle_distance(np.array([p]), a, b, c)[0]
        assert abs(got - want) < 1e-12, (p, got, want)


def test_chamfer_of_exact_plane_mesh_is_small():
    """A fine triangulation of the ground plane z = 0 of a one-plane scene: accuracy exactly 0 and
    completeness 0 for points on the plane inside it."""
    from voxelhashmt_gb300 import metrics, scenes
    sc = scenes.orbit_scene(seed=0, frames=1, width=8, height=8)
    sc.prims = sc.prims[:1]  # the ground plane z = 0 only
    g = np.linspace(-1.0, 1.0, 41)
    x, y = np.meshgrid(g, g)
    v = np.stack([x, y, np.zeros_like(x)], -1)
    t1 = np.stack([v[:-1, :-1], v[:-1, 1:], v[1:, :-1]], -2).reshape(-1, 9)
    t2 = np.stack([v[1:, 1:], v[1:, :-1], v[:-1, 1:]], -2).reshape(-1, 9)
    tris = np.concatenate([t1, t2]).astype(np.float32)
    rng = np.random.default_rng(1)
    pts = np.concatenate([rng.uniform(-0.9, 0.9, (500, 2)), np.zeros((500, 1))], 1)
    q = metrics.chamfer(tris, sc, pts)
    assert q["accuracy_mm"] < 1e-6 and q["completeness_mm"] < 1e-6, q
