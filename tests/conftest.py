"""Shared fixtures: the `gpu` marker, seeded scenes, and the built libraries."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def product_lib():
    from voxelhashmt_gb300 import build as pb
    pb.build()
    from voxelhashmt_gb300 import _capi
    _capi.lib()
    return _capi


@pytest.fixture(scope="session")
def small_orbit():
    """The orbit scene (plane, sphere, box) at 64x48 (focal length scaled with the resolution), 24 orbit poses, with the
    reference volume's default voxel size and truncation (voxel_hash_tsdf.h:191-192: 2 cm, 6 cm) so the
    oracle finishes in about a second."""
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=7, frames=24, width=64, height=48, fx=277.0 * 0.2, fy=277.0 * 0.2,
                            cx=32.0, cy=24.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    return sc


@pytest.fixture(scope="session")
def reference_demo(product_lib):
    """The reference's main.cpp + reconstruction_backend.cpp, unchanged, linked with the adapter
    (voxelhashmt_gb300/adapter) and libvoxelhash_gb300.so; built where the reference tree is present."""
    import subprocess
    from oracle import build as ob
    if not ob.reference_available():
        pytest.skip("reference tree not present")
    ref = ob.REFERENCE
    out_dir = os.path.join(ROOT, "oracle", "_ref")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "tsdf_demo_gb300")
    libdir = os.path.join(ROOT, "voxelhashmt_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-DTSDFMC_HAVE_CUDA=1",
           "-I", os.path.join(ref, "include"), "-I", os.path.join(ref, "src"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ref, "src", "main.cpp"), os.path.join(ref, "src", "reconstruction_backend.cpp"),
           os.path.join(ROOT, "voxelhashmt_gb300", "adapter", "tsdfmc_gb300_adapter.cpp"),
           "-L", libdir, "-lvoxelhash_gb300", "-Wl,-rpath," + libdir, "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return exe
