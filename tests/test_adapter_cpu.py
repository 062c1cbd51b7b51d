"""The reference-side binding: the reference's own main.cpp and reconstruction_backend.cpp, unchanged, link
against voxelhashmt_gb300/adapter/tsdfmc_gb300_adapter.cpp and libvoxelhash_gb300.so in place of the
reference's three .cu files.  Runs where the reference tree is present; the demo runs its CPU backend, and
its GPU backend reports the missing device through the C ABI when there is no GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_root():
    from oracle import build as ob
    return ob.REFERENCE if ob.reference_available() else None


@pytest.fixture(scope="module")
def demo(product_lib):
    ref = _reference_root()
    if ref is None:
        pytest.skip("reference tree not present")
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


def test_reference_demo_links_against_the_gb300_library(demo):
    nm = subprocess.run(["nm", "-C", demo], capture_output=True, text=True).stdout
    assert "tsdfmc::integrateDepthFrameCuda" in nm and "tsdfmc::extractMeshCuda" in nm
    ldd = subprocess.run(["ldd", demo], capture_output=True, text=True).stdout
    assert "libvoxelhash_gb300.so" in ldd


def test_reference_demo_gpu_backend_goes_through_the_c_abi(demo, tmp_path):
    torch = pytest.importorskip("torch")
    out = os.path.join(ROOT, "oracle", "_ref", "demo_out.ply")
    res = subprocess.run([demo, "--synthetic", "--backend", "gpu", "--frames", "2", "--width", "32", "--height", "24",
                          "--voxel-size", "0.02", "--truncation", "0.06", "--output", out],
                         capture_output=True, text=True, timeout=300)
    if torch.cuda.is_available():
        assert res.returncode == 0, res.stderr
        assert "GPU (CUDA)" in res.stdout and "raw triangles=" in res.stdout
    else:
        assert res.returncode == 1
        assert "GPU backend requested but CUDA is unavailable" in res.stderr
