"""The device renderer (vh_render_depth), which produces every benchmark and training frame, equals its host
restatement (the oracle's vo_render_depth) bit for bit, on several frames of each scene kind, with and without
noise.  The host restatement in turn follows the float64 renderer of scenes.py within stated bounds
(tests/test_oracle_cpu.py), and the reference arm of bench.py fuses frames from it: both arms fuse the same
frames."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libs(product_lib, oracle_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return product_lib, oracle_lib


def _device_render(capi, sc, frame, noise):
    K = sc.intrinsics
    prims = torch.from_numpy(np.ascontiguousarray(sc.prims, np.float32)).cuda()
    out = torch.empty((K.height, K.width), dtype=torch.float32, device="cuda")
    Kc, P = capi.intrinsics(K), capi.pose(sc.poses[frame])
    capi.check(capi.lib().vh_render_depth(C.c_void_p(prims.data_ptr()), prims.shape[0], C.byref(Kc), C.byref(P),
                                          sc.seed, frame, sc.noise_sigma_z2 if noise else 0.0,
                                          sc.dropout if noise else 0.0, sc.max_depth, C.c_void_p(out.data_ptr()),
                                          None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("kind", ["orbit", "room", "object_scan"])
def test_device_renderer_equals_host_restatement(libs, kind):
    capi, O = libs
    from voxelhashmt_gb300 import scenes
    sc = {"orbit": lambda: scenes.orbit_scene(seed=3, frames=64),
          "room": lambda: scenes.room_scene(seed=1, frames=40),
          "object_scan": lambda: scenes.object_scan_scene(seed=5)}[kind]()
    for frame in (0, 7, len(sc.poses) - 1):
        for noise in (True, False):
            got = _device_render(capi, sc, frame, noise)
            want = O.render_depth(sc, frame, noise=noise)
            assert (want > 0).sum() > 1000
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (kind, frame, noise)
