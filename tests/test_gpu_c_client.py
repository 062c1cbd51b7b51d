"""Native host code on the GPU: tests/capi_fuse_client.c, a pedantic C99 program linked against
libvoxelhash_gb300.so, fuses host depth frames and meshes the volume through the C ABI alone.  Its block count,
observed-voxel count and triangle soup equal the Python path's (TsdfIntegrationBackend over the same ABI) and
the oracle's, bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_c_client_fuses_and_meshes_like_the_python_path(product_lib, oracle_lib, small_orbit, tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if shutil.which("gcc") is None:
        pytest.skip("gcc not present")
    from voxelhashmt_gb300 import backend, scenes
    O = oracle_lib
    sc = small_orbit
    K = sc.intrinsics
    frames = [0, 5, 10, 15]
    buckets, max_blocks = 1 << 14, 4096
    data = bytearray()
    data += np.array([K.width, K.height, len(frames)], np.int32).tobytes()
    data += np.array([K.fx, K.fy, K.cx, K.cy, sc.voxel_size, sc.truncation], np.float32).tobytes()
    data += np.array([buckets, max_blocks], np.uint32).tobytes()
    depths = [scenes.render_depth(sc, f) for f in frames]
    for f, d in zip(frames, depths):
        data += np.asarray(sc.poses[f].as12(), np.float32).tobytes() + np.ascontiguousarray(d, np.float32).tobytes()
    fin, fout = os.path.join(str(tmp_path), "frames.bin"), os.path.join(str(tmp_path), "out.bin")
    with open(fin, "wb") as fh:
        fh.write(bytes(data))
    lib_dir = os.path.dirname(product_lib.LIB_PATH)
    exe = os.path.join(str(tmp_path), "capi_fuse_client")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "capi_fuse_client.c"), "-L", lib_dir, "-lvoxelhash_gb300",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True, capture_output=True)
    res = subprocess.run([exe, fin, fout], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    raw = open(fout, "rb").read()
    blocks, observed, ntri = np.frombuffer(raw[:24], np.uint64)
    soup = np.frombuffer(raw[24:], np.float32).reshape(int(ntri), 9)
    assert ntri > 1000

    vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=buckets, max_blocks=max_blocks)
    bk = backend.TsdfIntegrationBackend("gpu")
    ora = O.Volume(O.config(O.FLAVOR_REF_GPU, O.EXP_OWN, threads=8), sc.voxel_size, sc.truncation)
    for f, d in zip(frames, depths):
        bk.integrate(vol, backend.DepthFrame(K, d), sc.poses[f], 1)
        ora.integrate(d, K, sc.poses[f])
    tris = bk.extract_mesh(vol)
    assert int(blocks) == vol.block_count() == ora.block_count()
    assert int(observed) == vol.observed_voxel_count() == ora.observed_voxels()
    canon = O.canonical_triangles(soup).view(np.uint32)
    assert np.array_equal(canon, O.canonical_triangles(tris).view(np.uint32))
    assert np.array_equal(canon, O.canonical_triangles(ora.extract_mesh()).view(np.uint32))
    vol.close()
    ora.close()
