"""The device exponential (vh_expf) is the C library's expf.

* On the device, for all 2^32 float bit patterns, the fast single-precision path returns the same float as the
  C library's double-precision sequence (vh_expf_check): the fast path never changes a result.
* The device results equal the oracle's host restatement (vo_expf_own) bit for bit on a seeded sample of bit
  patterns and on every non-positive float in [-20, 0] of a stride.
* The restatement is the x86-64 GNU C library's expf (glibc 2.39, the host the reference was compiled and
  pinned on: equal on every float).  Other builds of the same algorithm differ from it only where the
  reduction step r = x * 32/ln2 - k is not fused into one multiply-add: at two arguments, -0x1.f8cbb2p+5 and
  0x1.04845ep+5.  On this host the C library may differ at the non-positive one of them and nowhere else.
"""
import ctypes as C
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libs(product_lib, oracle_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return product_lib, oracle_lib


def test_fast_path_equals_double_sequence_on_every_float(libs):
    capi, _ = libs
    L = capi.lib()
    n, first = C.c_uint64(), C.c_uint32()
    for lo in (0, 1 << 31):
        capi.check(L.vh_expf_check(lo, 1 << 31, C.byref(n), C.byref(first), None))
        assert n.value == 0, "%d differing arguments, the first %08x" % (n.value, first.value)


def _device_exp(capi, x):
    xd = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    yd = torch.empty_like(xd)
    capi.check(capi.lib().vh_expf_eval(C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), xd.numel(), None))
    torch.cuda.synchronize()
    return yd.cpu().numpy()


def test_device_exp_equals_host_restatement(libs):
    capi, O = libs
    rng = np.random.default_rng(5)
    bits = np.concatenate([
        rng.integers(0, 1 << 32, size=1 << 22, dtype=np.uint64).astype(np.uint32),
        np.arange(int(np.float32(-20.0).view(np.uint32)), int(np.float32(-0.0).view(np.uint32)) - 1, -97,
                  dtype=np.int64).astype(np.uint32),
        np.array([0x00000000, 0x80000000, 0x7f800000, 0xff800000, 0xc2cff1b4, 0xc2cff1b5, 0x42b17217, 0x42b17218],
                 np.uint32),
    ])
    x = bits.view(np.float32)
    got = _device_exp(capi, x)
    want = O.expf_array(x)
    nan = np.isnan(x)
    assert np.array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))
    assert np.isnan(got[nan]).all()


# the non-positive argument where an unfused reduction step rounds differently (the only one)
UNFUSED_REDUCTION_ARGUMENT = 0xC27C65D9


def test_host_c_library_expf_is_the_restatement(libs):
    """On this (GPU) host, the C library's expf equals the restatement on every non-positive float, except at
    most at the one argument where an unfused reduction step rounds differently."""
    _, O = libs
    n, first = O.expf_compare_libm(0x80000000, 0x7F800001, threads=max(os.cpu_count() or 1, 1))
    assert n == 0 or (n == 1 and first == UNFUSED_REDUCTION_ARGUMENT), \
        "%d differing arguments, the first %08x" % (n, first)
