"""The reference-side binding: the reference's own main.cpp and reconstruction_backend.cpp, unchanged, link
against voxelhashmt_gb300/adapter/tsdfmc_gb300_adapter.cpp and libvoxelhash_gb300.so in place of the
reference's three .cu files.  Runs where the reference tree is present; the demo runs its CPU backend, and
its GPU backend reports the missing device through the C ABI when there is no GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def demo(reference_demo):
    return reference_demo


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
