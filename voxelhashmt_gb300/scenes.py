"""Seeded analytic scenes and a numpy depth ray-caster for the depth-fusion path.

The reference renders its demo depth on the CPU by ray casting a sphere and a box
(src/main.cpp:189-335: ray-sphere, ray-AABB, depth = camera-space z, then noise and dropouts).
This module generates the workloads the fusion path is measured on with the same recipe:

* ``orbit_scene`` -- ground plane z=0, a sphere r=0.5 m and an axis-aligned box 0.4x0.3x0.6 m
  with seeded centres in a 1 m cube; the camera orbits at radius 1.5 m, height 0.8 m, looking
  at the origin; 320x240, fx=fy=277, cx=160, cy=120.
* ``room_scene`` -- the inside of a 4x5x3 m box room holding seeded spheres (r 0.1-0.6 m),
  boxes (0.1-1 m sides) and vertical cylinders; a hand-held random walk (1 cm/frame
  translation, 1 degree/frame yaw/pitch jitter); 640x480, fx=fy=525, cx=319.5, cy=239.5.
* ``multi_room_scene`` -- the large streaming configuration: a 20x20x4 m floor of 4x4 rooms (5x5 m,
  0.1 m walls with 1 m door gaps) holding 400 primitives in all; the camera walks room to room
  through the doors (about 1.25 cm/frame over 6000 frames) sweeping its yaw; 1280x720,
  fx=fy=1050 (the room configuration's field of view), 3 mm voxels, 1.2 cm truncation, 2^22 buckets.

Noise model for both: depth += N(0, (0.0012 z^2)^2) and 1 % of pixels dropped to 0.

Camera convention (src/main.cpp:177-187): x right, y down, z forward; ``Pose`` maps camera to
world (R row-major, t = camera centre).  World is z-up here.

Primitive records are float32 rows of ``PRIM_FIELDS`` values so the same scene can be handed
to the CUDA renderer (voxelhashmt_gb300/csrc/render.cu) unchanged:
    [type, a0, a1, a2, b0, b1, b2, r, h, 0]
    type 0 plane      n=(a0,a1,a2), offset r  (points p with n.p = r)
    type 1 sphere     centre a, radius r
    type 2 box        min corner a, max corner b
    type 3 cylinder   base centre a, radius r, height h (axis +z)
    type 4 room       min corner a, max corner b, seen from the inside
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PRIM_FIELDS = 10
PLANE, SPHERE, BOX, CYLINDER, ROOM = 0, 1, 2, 3, 4


@dataclass
class Intrinsics:
    """math_types.h:200-207."""
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float

    def k4(self):
        return np.array([self.fx, self.fy, self.cx, self.cy], dtype=np.float32)


@dataclass
class Pose:
    """Camera-to-world rigid transform, math_types.h:180-198 (R row-major 3x3, t)."""
    R: np.ndarray = field(default_factory=lambda: np.eye(3, dtype=np.float32))
    t: np.ndarray = field(default_factory=lambda: np.zeros(3, dtype=np.float32))

    def as12(self):
        return np.concatenate([np.asarray(self.R, np.float32).reshape(9),
                               np.asarray(self.t, np.float32).reshape(3)]).astype(np.float32)


@dataclass
class Scene:
    prims: np.ndarray                 # (P, PRIM_FIELDS) float32
    intrinsics: Intrinsics
    poses: list                       # list[Pose]
    seed: int
    noise_sigma_z2: float = 0.0012    # sigma = k * z^2
    dropout: float = 0.01
    voxel_size: float = 0.01
    truncation: float = 0.04
    hash_buckets: int = 1 << 16
    name: str = ""
    max_depth: float = 4.0            # returns outside (0.1, max_depth) are dropped (src/main.cpp:328)


def look_at(eye, target, up=(0.0, 0.0, 1.0)) -> Pose:
    """Camera x right, y down, z forward (the convention of src/main.cpp:177-187, with a z-up world)."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    R = np.stack([r, d, f], axis=1)
    return Pose(R.astype(np.float32), eye.astype(np.float32))


def _prim(kind, a=(0, 0, 0), b=(0, 0, 0), r=0.0, h=0.0):
    return [float(kind), *map(float, a), *map(float, b), float(r), float(h), 0.0]


def orbit_scene(seed=0, frames=64, width=320, height=240, fx=277.0, fy=277.0, cx=160.0, cy=120.0,
                radius=1.5, cam_height=0.8) -> Scene:
    rng = np.random.default_rng(seed)
    sphere_c = rng.uniform([-0.5, -0.5, 0.0], [0.5, 0.5, 1.0])
    box_c = rng.uniform([-0.5, -0.5, 0.0], [0.5, 0.5, 1.0])
    half = np.array([0.2, 0.15, 0.3])
    prims = [
        _prim(PLANE, (0, 0, 1), r=0.0),
        _prim(SPHERE, sphere_c, r=0.5),
        _prim(BOX, box_c - half, box_c + half),
    ]
    K = Intrinsics(width, height, fx, fy, cx, cy)
    poses = []
    for i in range(frames):
        a = 2.0 * math.pi * i / max(1, frames)
        eye = (radius * math.cos(a), radius * math.sin(a), cam_height)
        poses.append(look_at(eye, (0.0, 0.0, 0.0)))
    return Scene(np.asarray(prims, np.float32), K, poses, seed, name="orbit",
                 voxel_size=0.01, truncation=0.04, hash_buckets=1 << 16, max_depth=4.0)


def object_scan_scene(seed=0, frames=None, resolution=None, voxel_size=None) -> Scene:
    """One object scan of the batched multi-scene workload: a seeded cluster of 3-8 primitives (spheres r
    0.1-0.3 E, boxes 0.15-0.5 E sides, cylinders) within an extent E drawn from 0.5-2 m, resting on nothing
    (background returns no depth), seen by a camera orbiting once at 1.6 E + 0.4 m, 0.6 E above the cluster
    centre.  Frame count uniform in 20-300, resolution one of 160x120, 320x240, 640x480 (fx = fy = 0.866 W,
    a 60 degree horizontal field of view), voxel size uniform in 2-8 mm, truncation 4 voxels; each drawn from
    the seed unless given."""
    rng = np.random.default_rng(10_000 + seed)
    extent = float(rng.uniform(0.5, 2.0))
    n = int(rng.integers(3, 9))
    prims = []
    for _ in range(n):
        kind = int(rng.integers(0, 3))
        c = rng.uniform(-0.35, 0.35, size=3) * extent
        if kind == 0:
            prims.append(_prim(SPHERE, c, r=float(rng.uniform(0.1, 0.3) * extent)))
        elif kind == 1:
            half = rng.uniform(0.075, 0.25, size=3) * extent
            prims.append(_prim(BOX, c - half, c + half))
        else:
            r = float(rng.uniform(0.05, 0.2) * extent)
            h = float(rng.uniform(0.2, 0.7) * extent)
            prims.append(_prim(CYLINDER, (c[0], c[1], c[2] - h / 2), r=r, h=h))
    n_frames = int(rng.integers(20, 301)) if frames is None else int(frames)
    w, h = [(160, 120), (320, 240), (640, 480)][int(rng.integers(0, 3))] if resolution is None else resolution
    vs = float(rng.uniform(0.002, 0.008)) if voxel_size is None else float(voxel_size)
    K = Intrinsics(w, h, 0.866 * w, 0.866 * w, (w - 1) / 2.0, (h - 1) / 2.0)
    radius, height = 1.6 * extent + 0.4, 0.6 * extent
    phase = float(rng.uniform(0, 2 * math.pi))
    poses = []
    for i in range(n_frames):
        a = phase + 2.0 * math.pi * i / n_frames
        poses.append(look_at((radius * math.cos(a), radius * math.sin(a), height), (0.0, 0.0, 0.0)))
    sc = Scene(np.asarray(prims, np.float32), K, poses, seed, name="object_scan", voxel_size=vs, truncation=4 * vs,
               hash_buckets=1 << 18, max_depth=radius + 2 * extent)
    sc.extent = extent
    return sc


def room_scene(seed=0, frames=1000, width=640, height=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5,
               n_prims=40, room=(4.0, 5.0, 3.0)) -> Scene:
    rng = np.random.default_rng(seed)
    lo = np.zeros(3)
    hi = np.asarray(room, np.float64)
    start = np.array([hi[0] / 2, hi[1] / 2, 1.5])
    prims = [_prim(ROOM, lo, hi)]
    placed = 0
    while placed < n_prims:
        kind = rng.integers(0, 3)
        c = rng.uniform(lo + 0.2, hi - 0.2)
        if kind == 0:
            r = rng.uniform(0.1, 0.6)
            if np.linalg.norm(c - start) < r + 0.9:
                continue
            prims.append(_prim(SPHERE, c, r=r))
        elif kind == 1:
            s = rng.uniform(0.1, 1.0, size=3)
            if np.linalg.norm(c - start) < 0.9 + np.linalg.norm(s) / 2:
                continue
            prims.append(_prim(BOX, c - s / 2, c + s / 2))
        else:
            r = rng.uniform(0.08, 0.4)
            h = rng.uniform(0.3, 2.0)
            base = np.array([c[0], c[1], 0.0])
            if np.linalg.norm((c - start)[:2]) < r + 0.9:
                continue
            prims.append(_prim(CYLINDER, base, r=r, h=min(h, hi[2])))
        placed += 1
    K = Intrinsics(width, height, fx, fy, cx, cy)
    poses = []
    pos = start.copy()
    yaw = rng.uniform(0, 2 * math.pi)
    pitch = 0.0
    step = 0.01
    jitter = math.radians(1.0)
    for _ in range(frames):
        fwd = np.array([math.cos(pitch) * math.cos(yaw), math.cos(pitch) * math.sin(yaw), math.sin(pitch)])
        poses.append(look_at(pos, pos + fwd))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        pos = np.clip(pos + step * d, start - 0.5, start + 0.5)
        yaw += rng.uniform(-jitter, jitter)
        pitch = float(np.clip(pitch + rng.uniform(-jitter, jitter), -0.5, 0.5))
    return Scene(np.asarray(prims, np.float32), K, poses, seed, name="room",
                 voxel_size=0.005, truncation=0.02, hash_buckets=1 << 20, max_depth=8.0)


def multi_room_scene(seed=0, frames=6000, width=1280, height=720, fx=1050.0, fy=1050.0, cx=639.5, cy=359.5,
                     n_prims=400, rooms=4, room_size=5.0, height_m=4.0, door=1.0, wall=0.1) -> Scene:
    """A rooms x rooms grid of room_size rooms inside one shell: interior walls are boxes with a door gap
    (full height) in the middle of every room side, the rest of the n_prims primitives are seeded spheres,
    boxes and cylinders kept clear of the walk and the walls.  The walk visits the rooms in serpentine order,
    room centre -> door -> next room centre, at 1.5 m height; the camera looks along the walk with a slow
    +-50 degree yaw sweep and small pitch jitter."""
    rng = np.random.default_rng(seed)
    side = rooms * room_size
    prims = [_prim(ROOM, (0.0, 0.0, 0.0), (side, side, height_m))]
    hw = wall / 2
    for k in range(1, rooms):  # interior wall lines x = k * room_size and y = k * room_size
        w = k * room_size
        for j in range(rooms):
            a, b = j * room_size, (j + 1) * room_size
            mid = (a + b) / 2
            for lo_, hi_ in ((a, mid - door / 2), (mid + door / 2, b)):
                prims.append(_prim(BOX, (w - hw, lo_, 0.0), (w + hw, hi_, height_m)))
                prims.append(_prim(BOX, (lo_, w - hw, 0.0), (hi_, w + hw, height_m)))
    # the walk: serpentine over the room grid, through the door in the shared wall
    order = []
    for row in range(rooms):
        cols = range(rooms) if row % 2 == 0 else range(rooms - 1, -1, -1)
        order += [(c, row) for c in cols]

    def centre(c, r):
        return np.array([(c + 0.5) * room_size, (r + 0.5) * room_size, 1.5])

    way = [centre(*order[0])]
    for (c0, r0), (c1, r1) in zip(order, order[1:]):
        way.append((centre(c0, r0) + centre(c1, r1)) / 2)  # the door between two adjacent rooms
        way.append(centre(c1, r1))
    way = np.asarray(way)
    seg = np.linalg.norm(np.diff(way, axis=0), axis=1)
    cum = np.concatenate([[0.0], np.cumsum(seg)])

    def clear_of_walk(p, r):
        for a, b in zip(way[:-1], way[1:]):
            ab = b - a
            t = np.clip(np.dot(p[:2] - a[:2], ab[:2]) / max(np.dot(ab[:2], ab[:2]), 1e-9), 0.0, 1.0)
            if np.linalg.norm(p[:2] - (a[:2] + t * ab[:2])) < r + 0.7:
                return False
        return True

    def clear_of_walls(p, r):
        for k in range(1, rooms):
            w = k * room_size
            if abs(p[0] - w) < r + hw + 0.05 or abs(p[1] - w) < r + hw + 0.05:
                return False
        return True

    placed = len(prims)
    while placed < n_prims:
        kind = rng.integers(0, 3)
        c = np.array([rng.uniform(0.3, side - 0.3), rng.uniform(0.3, side - 0.3), rng.uniform(0.2, height_m - 0.5)])
        if kind == 0:
            r = rng.uniform(0.1, 0.5)
            if not (clear_of_walk(c, r) and clear_of_walls(c, r)):
                continue
            prims.append(_prim(SPHERE, c, r=r))
        elif kind == 1:
            s = rng.uniform(0.1, 0.9, size=3)
            rr = float(np.linalg.norm(s[:2])) / 2
            if not (clear_of_walk(c, rr) and clear_of_walls(c, rr)):
                continue
            prims.append(_prim(BOX, c - s / 2, c + s / 2))
        else:
            r = rng.uniform(0.08, 0.35)
            h = rng.uniform(0.3, 2.5)
            base = np.array([c[0], c[1], 0.0])
            if not (clear_of_walk(base, r) and clear_of_walls(base, r)):
                continue
            prims.append(_prim(CYLINDER, base, r=r, h=min(h, height_m)))
        placed += 1
    K = Intrinsics(width, height, fx, fy, cx, cy)
    poses = []
    s_at = np.linspace(0.0, cum[-1], frames)
    jitter = math.radians(1.0)
    pitch = 0.0
    for i, sv in enumerate(s_at):
        k = min(int(np.searchsorted(cum, sv, side="right")) - 1, len(seg) - 1)
        t = (sv - cum[k]) / seg[k]
        pos = way[k] + t * (way[k + 1] - way[k])
        d = way[k + 1] - way[k]
        yaw = math.atan2(d[1], d[0]) + math.radians(50.0) * math.sin(2 * math.pi * i / 600.0)
        pitch = float(np.clip(pitch + rng.uniform(-jitter, jitter), -0.3, 0.3))
        fwd = np.array([math.cos(pitch) * math.cos(yaw), math.cos(pitch) * math.sin(yaw), math.sin(pitch)])
        poses.append(look_at(pos, pos + fwd))
    return Scene(np.asarray(prims, np.float32), K, poses, seed, name="multi_room",
                 voxel_size=0.003, truncation=0.012, hash_buckets=1 << 22, max_depth=8.0)


def _hash_u32(x):
    """lowbias32 integer hash (public domain, C. Wellons); uint32 in, uint32 out."""
    x = np.asarray(x, np.uint32)
    x = x ^ (x >> np.uint32(16))
    x = (x * np.uint32(0x7FEB352D)).astype(np.uint32)
    x = x ^ (x >> np.uint32(15))
    x = (x * np.uint32(0x846CA68B)).astype(np.uint32)
    x = x ^ (x >> np.uint32(16))
    return x


def _uniforms(seed, frame, n, stream):
    idx = np.arange(n, dtype=np.uint32)
    key = np.uint32((seed * 0x9E3779B1 + frame * 0x85EBCA77 + stream * 0xC2B2AE3D) & 0xFFFFFFFF)
    h = _hash_u32(idx ^ _hash_u32(np.full(n, key, np.uint32)))
    return (h.astype(np.float64) + 0.5) / 4294967296.0


def _intersect(prims, o, d):
    """Nearest positive hit distance along unit rays d (N,3) from origin o (3,)."""
    n = d.shape[0]
    best = np.full(n, np.inf)
    eps = 1e-4
    for p in prims:
        kind = int(p[0])
        a = p[1:4].astype(np.float64)
        b = p[4:7].astype(np.float64)
        r = float(p[7])
        h = float(p[8])
        if kind == PLANE:
            denom = d @ a
            with np.errstate(divide="ignore", invalid="ignore"):
                t = (r - o @ a) / denom
            t[~np.isfinite(t) | (t <= eps)] = np.inf
        elif kind == SPHERE:
            oc = o - a
            bb = d @ oc
            c = oc @ oc - r * r
            disc = bb * bb - c
            sq = np.sqrt(np.maximum(disc, 0.0))
            t0 = -bb - sq
            t1 = -bb + sq
            t = np.where(t0 > eps, t0, t1)
            t[(disc < 0) | (t <= eps)] = np.inf
        elif kind in (BOX, ROOM):
            with np.errstate(divide="ignore", invalid="ignore"):
                inv = 1.0 / d
                ta = (a - o) * inv
                tb = (b - o) * inv
            tmin = np.nanmax(np.minimum(ta, tb), axis=1)
            tmax = np.nanmin(np.maximum(ta, tb), axis=1)
            if kind == BOX:
                t = np.where(tmin > eps, tmin, tmax)
                t[(tmax < tmin) | (tmax <= eps)] = np.inf
            else:
                t = tmax.copy()
                t[t <= eps] = np.inf
        elif kind == CYLINDER:
            ox, oy = o[0] - a[0], o[1] - a[1]
            dx, dy = d[:, 0], d[:, 1]
            qa = dx * dx + dy * dy
            qb = ox * dx + oy * dy
            qc = ox * ox + oy * oy - r * r
            disc = qb * qb - qa * qc
            with np.errstate(divide="ignore", invalid="ignore"):
                sq = np.sqrt(np.maximum(disc, 0.0))
                t0 = (-qb - sq) / qa
                t1 = (-qb + sq) / qa
            t = np.full(n, np.inf)
            for tc in (t1, t0):
                z = o[2] + tc * d[:, 2]
                ok = (disc >= 0) & (tc > eps) & (z >= a[2]) & (z <= a[2] + h) & (qa > 1e-12)
                t = np.where(ok, tc, t)
            # caps
            for zc in (a[2], a[2] + h):
                with np.errstate(divide="ignore", invalid="ignore"):
                    tc = (zc - o[2]) / d[:, 2]
                px = ox + tc * dx
                py = oy + tc * dy
                ok = np.isfinite(tc) & (tc > eps) & (px * px + py * py <= r * r)
                t = np.where(ok & (tc < t), tc, t)
        else:
            raise ValueError(kind)
        best = np.minimum(best, t)
    return best


def render_depth(scene: Scene, frame: int, noise=True) -> np.ndarray:
    """Ray-cast depth (camera z, metres, float32 HxW, 0 = no return) for one frame."""
    K = scene.intrinsics
    P = scene.poses[frame]
    u, v = np.meshgrid(np.arange(K.width, dtype=np.float64), np.arange(K.height, dtype=np.float64))
    dc = np.stack([(u - K.cx) / K.fx, (v - K.cy) / K.fy, np.ones_like(u)], axis=-1).reshape(-1, 3)
    dc /= np.linalg.norm(dc, axis=1, keepdims=True)
    R = np.asarray(P.R, np.float64)
    dw = dc @ R.T
    t = _intersect(scene.prims, np.asarray(P.t, np.float64), dw)
    z = t * dc[:, 2]
    z[~np.isfinite(z)] = 0.0
    if noise:
        n = z.shape[0]
        u1 = _uniforms(scene.seed, frame, n, 0)
        u2 = _uniforms(scene.seed, frame, n, 1)
        g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)
        z = z + g * scene.noise_sigma_z2 * z * z
        drop = _uniforms(scene.seed, frame, n, 2) < scene.dropout
        z[drop] = 0.0
    z[(z < 0.1) | (z > scene.max_depth)] = 0.0
    return z.reshape(K.height, K.width).astype(np.float32)


def scene_sdf(prims: np.ndarray, pts: np.ndarray) -> np.ndarray:
    """Unsigned distance from points (N,3) to the union of the scene's analytic surfaces."""
    pts = np.asarray(pts, np.float64)
    best = np.full(pts.shape[0], np.inf)
    for p in prims:
        kind = int(p[0])
        a = p[1:4].astype(np.float64)
        b = p[4:7].astype(np.float64)
        r = float(p[7])
        h = float(p[8])
        if kind == PLANE:
            dist = np.abs(pts @ a - r)
        elif kind == SPHERE:
            dist = np.abs(np.linalg.norm(pts - a, axis=1) - r)
        elif kind in (BOX, ROOM):
            c = (a + b) / 2
            e = (b - a) / 2
            q = np.abs(pts - c) - e
            outside = np.linalg.norm(np.maximum(q, 0.0), axis=1)
            inside = np.minimum(np.max(q, axis=1), 0.0)
            dist = np.abs(outside + inside)
        elif kind == CYLINDER:
            rr = np.linalg.norm(pts[:, :2] - a[:2], axis=1) - r
            zz = np.abs(pts[:, 2] - (a[2] + h / 2)) - h / 2
            q = np.stack([rr, zz], axis=1)
            dist = np.abs(np.linalg.norm(np.maximum(q, 0.0), axis=1) + np.minimum(np.max(q, axis=1), 0.0))
        else:
            raise ValueError(kind)
        best = np.minimum(best, dist)
    return best
