"""GPU tests of the denoiser's tensor-core convolution (vh_nn_conv32) against a float64 PyTorch reference on
the same BF16-rounded operands.  Tolerance: one BF16 unit in the last place of the reference value (the
kernel accumulates in FP32 and rounds once to BF16), plus 1e-6 absolute."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi(product_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return product_lib


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _conv_ref(x_nhwc, w, bias):
    """x: (B, H, W, 32) float64, w: (32, 32, 3, 3) float64 -> (B, H, W, 32) float64, zero padding."""
    import torch.nn.functional as F
    y = F.conv2d(x_nhwc.permute(0, 3, 1, 2), w, bias, padding=1)
    return y.permute(0, 2, 3, 1)


def _run(capi, x_bf, w32, bias, mask_bf, mode, relu, transpose_flip=0):
    packed = torch.empty(9 * 32 * 32, dtype=torch.bfloat16, device="cuda")
    capi.check(capi.lib().vh_nn_pack_conv32_weights(_ptr(w32), _ptr(packed), transpose_flip, None))
    out = torch.full_like(x_bf, float("nan"))
    err = C.c_uint32(0)
    err_dev = torch.zeros(1, dtype=torch.int32, device="cuda")
    B, H, W, _ = x_bf.shape
    capi.check(capi.lib().vh_nn_conv32(_ptr(x_bf), _ptr(packed), _ptr(bias) if bias is not None else None,
                                       _ptr(mask_bf) if mask_bf is not None else None, _ptr(out), B, W, H, mode, relu,
                                       C.cast(C.c_void_p(err_dev.data_ptr()), C.POINTER(C.c_uint32)), None))
    torch.cuda.synchronize()
    assert int(err_dev.item()) == 0, "tensor cores did not signal completion"
    return out


def _close(got_bf, ref64):
    got = got_bf.double().cpu()
    ref = ref64.cpu()
    ulp = torch.clamp(ref.abs(), min=1e-30) * 2.0 ** -7
    bad = (got - ref).abs() > ulp + 1e-6
    return int(bad.sum()), float((got - ref).abs().max())


@pytest.mark.parametrize("shape", [(1, 3, 128), (2, 5, 200), (1, 17, 331)])
def test_conv32_forward_matches_reference(capi, shape):
    B, H, W = shape
    g = torch.Generator().manual_seed(B * 1000 + H * 10 + W)
    x = torch.randn(B, H, W, 32, generator=g).to(torch.bfloat16).cuda().contiguous()
    w = (torch.randn(32, 32, 3, 3, generator=g) * 0.1).float().cuda().contiguous()
    b = (torch.randn(32, generator=g) * 0.1).float().cuda().contiguous()
    wq = w.to(torch.bfloat16).double()
    for relu in (0, 1):
        out = _run(capi, x, w, b, None, 0, relu)
        ref = _conv_ref(x.double(), wq, b.double())
        if relu:
            ref = torch.clamp(ref, min=0.0)
        nbad, worst = _close(out, ref)
        assert nbad == 0, (nbad, worst)


def test_conv32_input_gradient_matches_reference(capi):
    """mode 1 with transposed, flipped weights: the input gradient of a 3x3 convolution, masked by ReLU."""
    B, H, W = 2, 9, 150
    g = torch.Generator().manual_seed(7)
    dy = torch.randn(B, H, W, 32, generator=g).to(torch.bfloat16).cuda().contiguous()
    act = torch.randn(B, H, W, 32, generator=g).to(torch.bfloat16).cuda().contiguous()
    w = (torch.randn(32, 32, 3, 3, generator=g) * 0.1).float().cuda().contiguous()
    out = _run(capi, dy, w, None, act, 1, 0, transpose_flip=1)
    # reference: d/dx of sum(conv(x, w) * dy) = conv_transpose(dy, w), then the ReLU mask of act
    import torch.nn.functional as F
    wq = w.to(torch.bfloat16).double()
    ref = F.conv_transpose2d(dy.double().permute(0, 3, 1, 2), wq, padding=1).permute(0, 2, 3, 1)
    ref = torch.where(act.double() > 0, ref, torch.zeros_like(ref))
    nbad, worst = _close(out, ref)
    assert nbad == 0, (nbad, worst)
