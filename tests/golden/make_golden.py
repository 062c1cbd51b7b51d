"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference build (oracle/_ref/libref.so, made by `python oracle/build.py --ref` from the reference
sources: the CPU path compiled as-is and the CUDA kernels compiled for the host under the emulation prelude)
on a small seeded scene, and stores inputs and outputs:

  golden_scene.npz     depth frames (48x36, 3 frames), poses, intrinsics, voxel size, truncation
  golden_gpu.npz       the reference CUDA path (emulated, C library expf): filtered depth of frame 0, the
                       block keys allocateActiveBlocksCuda returns for frame 0 (raw depth, stride 1 and 2),
                       after integrating the 3 frames: sorted block keys, observed-voxel count, SHA-256 of the
                       sorted voxel bytes, the voxels of the 4 fullest blocks, and the sorted triangle soup
  golden_cpu.npz       the same for the reference CPU path (TsdfIntegrationBackend(kCpu))
  golden_kat.npz       known answers of hashBlockKey / packBlockKey, the GPU and CPU octahedral packers and
                       unpackers, and computeObservationWeightGpu on seeded random inputs

usage: python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as ob  # noqa: E402
from oracle import oracle as O  # noqa: E402
from voxelhashmt_gb300 import scenes  # noqa: E402


def golden_scene():
    sc = scenes.orbit_scene(seed=1234, frames=12, width=48, height=36, fx=41.6, fy=41.6, cx=24.0, cy=18.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    frames = [0, 4, 8]
    return sc, frames


def voxel_digest(vox):
    return hashlib.sha256(np.ascontiguousarray(vox).view(np.uint8).tobytes()).hexdigest()


def fullest(keys, vox, n=4):
    w = vox["weight"].reshape(vox.shape[0], -1)
    counts = (w > 0).sum(axis=1)
    idx = np.sort(np.argsort(-counts, kind="stable")[:n])
    return keys[idx], vox[idx]


def run_flavor(sc, frames, gpu):
    K = sc.intrinsics
    d0 = scenes.render_depth(sc, frames[0])
    out = {
        "filtered0": O.ref_filter(d0, K, gpu),
        "keys_stride1": O.ref_collect(d0, K, sc.poses[frames[0]], sc.voxel_size, sc.truncation, 1, gpu),
        "keys_stride2": O.ref_collect(d0, K, sc.poses[frames[0]], sc.voxel_size, sc.truncation, 2, gpu),
    }
    vol = O.RefVolume(gpu, sc.voxel_size, sc.truncation)
    for f in frames:
        vol.integrate(scenes.render_depth(sc, f), K, sc.poses[f])
    keys, vox = O.sort_blocks(*vol.blocks())
    out["block_keys"] = keys
    out["observed_voxels"] = np.int64(vol.observed_voxels())
    out["voxel_sha256"] = np.array(voxel_digest(vox))
    fk, fv = fullest(keys, vox)
    out["fullest_keys"] = fk
    out["fullest_voxels"] = fv.view(np.uint32)
    out["triangles"] = O.canonical_triangles(vol.extract_mesh())
    vol.close()
    return out


def kat():
    rng = np.random.default_rng(99)
    R = O.ref()
    import ctypes as C
    keys = rng.integers(-(1 << 20) - 4, (1 << 20) + 4, size=(512, 3)).astype(np.int32)
    keys[:8] = [[0, 0, 0], [-1, -1, -1], [(1 << 20) - 1, 0, 0], [-(1 << 20), 0, 0], [1 << 20, 0, 0],
                [0, -(1 << 20) - 1, 0], [5, -7, 11], [-123456, 654321, -1]]
    hashes = np.array([R.ref_gpu_hash_block_key(*map(int, k)) for k in keys], np.uint32)
    packed = np.zeros(len(keys), np.uint64)
    packable = np.zeros(len(keys), np.int32)
    for i, k in enumerate(keys):
        p = C.c_ulonglong()
        packable[i] = R.ref_gpu_pack_block_key(*map(int, k), C.byref(p))
        packed[i] = p.value if packable[i] else 0
    normals = rng.normal(size=(1024, 3)).astype(np.float32)
    normals[:6] = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]]
    normals[6] = [0, 0, 0]
    pack_gpu = np.array([R.ref_gpu_pack_normal(n.ctypes.data_as(C.POINTER(C.c_float))) for n in normals], np.uint32)
    pack_cpu = np.array([R.ref_cpu_pack_normal(n.ctypes.data_as(C.POINTER(C.c_float))) for n in normals], np.uint32)
    codes = np.concatenate([pack_gpu, rng.integers(0, 1 << 32, size=512, dtype=np.uint64).astype(np.uint32)])
    unpack = {}
    for name, fn in (("unpack_gpu", R.ref_gpu_unpack_normal), ("unpack_gpu_mesh", R.ref_gpu_mesh_unpack_normal),
                     ("unpack_cpu", R.ref_cpu_unpack_normal)):
        out = np.zeros((len(codes), 3), np.float32)
        for i, c in enumerate(codes):
            fn(int(c), out[i].ctypes.data_as(C.POINTER(C.c_float)))
        unpack[name] = out
    wargs = np.stack([rng.uniform(-0.5, 6.0, 1024), rng.uniform(-0.2, 0.2, 1024), rng.choice([0.0, 1e-7, 0.02, 0.06], 1024),
                      rng.uniform(-0.2, 1.2, 1024)], axis=1).astype(np.float32)
    weights = np.array([R.ref_gpu_observation_weight(*map(float, a)) for a in wargs], np.float32)
    return dict(keys=keys, hashes=hashes, packed=packed, packable=packable, normals=normals, pack_gpu=pack_gpu,
                pack_cpu=pack_cpu, codes=codes, weight_args=wargs, weights=weights, **unpack)


def main():
    ob.build_oracle()
    if ob.build_ref() is None:
        raise SystemExit("the reference tree is not available: cannot generate fixtures")
    sc, frames = golden_scene()
    K = sc.intrinsics
    np.savez_compressed(os.path.join(HERE, "golden_scene.npz"),
                        depth=np.stack([scenes.render_depth(sc, f) for f in frames]),
                        poses=np.stack([sc.poses[f].as12() for f in frames]),
                        intrinsics=np.array([K.width, K.height, K.fx, K.fy, K.cx, K.cy], np.float64),
                        voxel_size=np.float32(sc.voxel_size), truncation=np.float32(sc.truncation))
    for gpu, name in ((True, "golden_gpu.npz"), (False, "golden_cpu.npz")):
        np.savez_compressed(os.path.join(HERE, name), **run_flavor(sc, frames, gpu))
    np.savez_compressed(os.path.join(HERE, "golden_kat.npz"), **kat())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
