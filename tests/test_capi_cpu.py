"""The C ABI library without a GPU: it builds for sm_103a, loads, exports every function the public header
declares, carries the reference CUDA path's constants, and reports the missing device as a status."""
import ctypes as C

import pytest


def test_library_exports_every_header_function(product_lib):
    capi = product_lib
    declared = capi.header_symbols()
    assert "vh_integrate" in declared and "vh_extract_mesh" in declared and len(declared) >= 20
    lib = capi.lib()
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing
    assert set(capi._SIGNATURES) == set(declared), set(capi._SIGNATURES) ^ set(declared)


def test_default_constants_are_the_reference_gpu_constants(product_lib):
    a = product_lib.default_algorithm()
    # src/cuda_tsdf_integrator.cu:18-35, src/cuda_mesh_extractor.cu:20
    expect = dict(depth_discontinuity_base=0.012, depth_discontinuity_relative=0.025, filter_radius=2,
                  filter_sigma_spatial=1.5, filter_sigma_range=0.0012, filter_sigma_angular=0.35,
                  filter_min_cosine=0.9, normal_radius=1, normal_sigma_spatial=1.0, normal_sigma_range=0.0012,
                  normal_sigma_angular=0.35, layer_merge_voxel_scale=0.25, layer_normal_cosine=0.9,
                  layer_extract_voxel_scale=0.55, max_voxel_weight=100.0, depth_sigma=1.5, huber_delta=0.35,
                  min_observation_weight=0.05, min_view_angle_weight=0.15)
    for k, v in expect.items():
        assert getattr(a, k) == pytest.approx(v, rel=0, abs=0) if isinstance(v, int) else \
            C.c_float(getattr(a, k)).value == C.c_float(v).value, k


def test_status_strings_and_argument_checks(product_lib):
    capi = product_lib
    L = capi.lib()
    for s in range(0, 13):
        assert L.vh_status_string(s) != b"unknown status"
    h = C.c_void_p()
    bad = capi.default_params(hash_buckets=1000)  # not a power of two
    assert L.vh_create(C.byref(bad), None, C.byref(h)) == capi.VH_ERR_INVALID_ARGUMENT
    bad = capi.default_params(max_blocks=(1 << 23) + 1)
    assert L.vh_create(C.byref(bad), None, C.byref(h)) == capi.VH_ERR_INVALID_ARGUMENT
    # the checks come before any device call
    n1, n2 = C.c_size_t(), C.c_size_t()
    assert L.vh_weld_mesh(None, C.byref(n1), C.byref(n2), None) == capi.VH_ERR_INVALID_ARGUMENT
    assert L.vh_copy_welded_mesh(None, None, 0, None, 0, 0, None) == capi.VH_ERR_INVALID_ARGUMENT
    err = (C.c_uint32 * 1)()
    assert L.vh_nn_conv32_gated(None, None, None, None, None, 1, 8, 8, 0, 0, None, err, None) == \
        capi.VH_ERR_INVALID_ARGUMENT
    assert L.vh_nn_wgrad32(None, None, None, None, 1, 8, 8, err, None) == capi.VH_ERR_INVALID_ARGUMENT
    ev = C.c_uint64()
    assert L.vh_evict_blocks(None, 0, 0, 1, None, None, 0, 0, C.byref(ev), None) == capi.VH_ERR_INVALID_ARGUMENT
    assert L.vh_restore_blocks(None, None, None, 1, 0, None) == capi.VH_ERR_INVALID_ARGUMENT


def test_no_device_is_reported_not_faked(product_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    capi = product_lib
    L = capi.lib()
    buf = C.create_string_buffer(128)
    assert L.vh_query_device(buf, 128) == capi.VH_ERR_NO_DEVICE
    h = C.c_void_p()
    assert L.vh_create(C.byref(capi.default_params()), None, C.byref(h)) == capi.VH_ERR_NO_DEVICE
    from voxelhashmt_gb300 import backend
    with pytest.raises(RuntimeError):
        backend.TsdfIntegrationBackend("gpu")
    with pytest.raises(RuntimeError):
        backend.TsdfIntegrationBackend("cpu")  # no CPU path in the product


def test_backend_preference_parsing():
    from voxelhashmt_gb300 import backend
    assert backend.parse_compute_backend_preference("GPU") is backend.ComputeBackendPreference.GPU
    assert backend.parse_compute_backend_preference("auto") is backend.ComputeBackendPreference.AUTO
    with pytest.raises(ValueError):
        backend.parse_compute_backend_preference("tpu")


def test_header_is_plain_c_and_a_c_program_links(product_lib, tmp_path):
    """The boundary is a C ABI: the public header compiles as pedantic C99, and a C program linked against the
    library runs its device-free calls (defaults, status strings, the device query)."""
    import os
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not present")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib_dir = os.path.dirname(product_lib.LIB_PATH)
    src = os.path.join(str(tmp_path), "client.c")
    with open(src, "w") as f:
        f.write('#include <stdio.h>\n#include "voxelhash_gb300.h"\n'
                "int main(void) {\n"
                "  vh_params p; vh_algorithm a; char msg[128];\n"
                "  vh_params_default(&p); vh_algorithm_default(&a);\n"
                "  vh_status s = vh_query_device(msg, sizeof msg);\n"
                '  printf("%g %g %d %s|%s\\n", p.voxel_size, a.filter_sigma_spatial, (int)s, vh_status_string(s), '
                "msg);\n"
                "  return (p.voxel_size > 0.0f && a.filter_radius == 2) ? 0 : 1;\n"
                "}\n")
    exe = os.path.join(str(tmp_path), "client")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(root, "include"),
                    src, "-L", lib_dir, "-lvoxelhash_gb300", "-Wl,-rpath," + lib_dir, "-o", exe], check=True,
                   capture_output=True)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.startswith("0.01 1.5 ")
