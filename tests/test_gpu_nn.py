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


@pytest.mark.parametrize("shape", [(1, 3, 64), (2, 17, 150), (1, 35, 331), (3, 1, 7)])
def test_wgrad32_matches_reference(capi, shape):
    """vh_nn_wgrad32 (the weight and bias gradients of a 32 -> 32 layer on the tensor cores) against float64 on
    the same BF16 operands: partial strips and row blocks, a one-row image.  The products of BF16 values are exact
    in FP32; the tolerance covers FP32 accumulation in any order: 1e-5 of the sum of the terms' magnitudes."""
    B, H, W = shape
    g = torch.Generator().manual_seed(B * 7919 + H * 31 + W)
    x = torch.randn(B, H, W, 32, generator=g).to(torch.bfloat16)
    dy = torch.randn(B, H, W, 32, generator=g).to(torch.bfloat16)
    dw0 = torch.randn(32 * 32 * 9, generator=g).float()  # accumulated into
    db0 = torch.randn(32, generator=g).float()
    dw, db = dw0.clone().cuda(), db0.clone().cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    xd, gd = x.cuda().contiguous(), dy.cuda().contiguous()
    capi.check(capi.lib().vh_nn_wgrad32(_ptr(xd), _ptr(gd), _ptr(dw), _ptr(db), B, W, H,
                                        C.cast(C.c_void_p(err.data_ptr()), C.POINTER(C.c_uint32)), None))
    torch.cuda.synchronize()
    assert int(err.item()) == 0, "tensor cores did not signal completion"
    xn, gn = x.double().permute(0, 3, 1, 2), dy.double().permute(0, 3, 1, 2)
    ref = torch.nn.grad.conv2d_weight(xn, (32, 32, 3, 3), gn, padding=1).reshape(-1)
    mag = torch.nn.grad.conv2d_weight(xn.abs(), (32, 32, 3, 3), gn.abs(), padding=1).reshape(-1)
    got = dw.double().cpu() - dw0.double()
    bad = (got - ref).abs() > 1e-5 * mag + 1e-6 * (1.0 + dw0.double().abs())
    assert int(bad.sum()) == 0, (int(bad.sum()), float((got - ref).abs().max()))
    bref = gn.sum(dim=(0, 2, 3))
    bmag = gn.abs().sum(dim=(0, 2, 3))
    bgot = db.double().cpu() - db0.double()
    assert bool(((bgot - bref).abs() <= 1e-5 * bmag + 1e-6 * (1.0 + db0.double().abs())).all())


def _bf(t):
    """BF16 rounding in the forward pass, identity in the backward (straight-through)."""
    return t + (t.to(torch.bfloat16).double() - t).detach()


def _round_grad(t):
    t.register_hook(lambda g: g.to(torch.bfloat16).double())
    return t


def _ref_loss(params, depth, target):
    """The net in float64 on the CPU, BF16 rounding where the kernels store BF16: weights of the two 32 -> 32
    layers, the activations, and the activation gradients."""
    import torch.nn.functional as F
    sizes = [32 * 4 * 9, 32, 32 * 32 * 9, 32, 32 * 32 * 9, 32, 32 * 9, 1]
    w1, b1, w2, b2, w3, b3, w4, b4 = torch.split(params, sizes)
    d = depth.unsqueeze(1)
    valid = (d > 0).double()
    ones = torch.ones(1, 1, 3, 3, dtype=torch.float64)
    s = F.conv2d(d * valid, ones, padding=1)
    c = F.conv2d(valid, ones, padding=1)
    m = torch.where(c > 0, s / torch.clamp(c, min=1), torch.zeros_like(s))
    X = torch.cat([(d - m) * 100 * valid, valid, m * 0.25 * valid, torch.zeros_like(d)], 1)
    z1 = _round_grad(F.conv2d(X, w1.view(32, 4, 3, 3), b1, padding=1))
    a1 = _bf(torch.relu(z1))
    z2 = _round_grad(F.conv2d(a1, _bf(w2.view(32, 32, 3, 3)), b2, padding=1))
    a2 = _bf(torch.relu(z2))
    z3 = _round_grad(F.conv2d(a2, _bf(w3.view(32, 32, 3, 3)), b3, padding=1))
    a3 = _bf(torch.relu(z3))
    r = F.conv2d(a3, w4.view(1, 32, 3, 3), b4, padding=1)
    out = torch.where(valid > 0, torch.clamp(d + 0.01 * r, min=0.0), torch.zeros_like(d)).squeeze(1)
    gate = torch.clamp(0.025 * target, min=0.012)
    mask = (depth > 0) & (target > 0) & (out > 0) & ((depth - target).abs() <= gate)
    loss = torch.where(mask, (out - target) ** 2, torch.zeros_like(out)).sum() / out.numel()
    return loss, out


def test_denoiser_forward_and_gradients_match_reference(capi):
    """Forward output within 0.1 mm and every parameter group's gradient within 2 % (relative L2) of the
    float64 reference on the same BF16-rounded operands, on a batch of two 150 x 24 rooms crops (two tensor-
    core tiles per row, one partial)."""
    from voxelhashmt_gb300 import denoiser, scenes
    sc = scenes.room_scene(seed=3, frames=2, width=150, height=24, fx=120.0, fy=120.0, cx=75.0, cy=12.0)
    raw = np.stack([scenes.render_depth(sc, f) for f in range(2)]).astype(np.float32)
    tgt = np.stack([scenes.render_depth(sc, f, noise=False) for f in range(2)]).astype(np.float32)
    p0 = denoiser.init_params(seed=5)
    p0[-289:] = np.random.default_rng(6).normal(0, 0.05, 289).astype(np.float32)  # a non-trivial output layer
    net = denoiser.DepthDenoiser(p0)
    g_gpu, loss_gpu, out_gpu = net.gradients(torch.from_numpy(raw).cuda(), torch.from_numpy(tgt).cuda())
    params = torch.from_numpy(p0.astype(np.float64)).requires_grad_(True)
    loss_ref, out_ref = _ref_loss(params, torch.from_numpy(raw).double(), torch.from_numpy(tgt).double())
    loss_ref.backward()
    g_ref = params.grad.numpy()
    assert np.max(np.abs(out_gpu.cpu().numpy() - out_ref.detach().numpy())) <= 1e-4
    assert abs(loss_gpu - float(loss_ref)) <= 1e-3 * float(loss_ref) + 1e-12
    sizes = [32 * 4 * 9, 32, 32 * 32 * 9, 32, 32 * 32 * 9, 32, 32 * 9, 1]
    names = ["w1", "b1", "w2", "b2", "w3", "b3", "w4", "b4"]
    off = 0
    for name, n in zip(names, sizes):
        a, b = g_gpu[off:off + n].astype(np.float64), g_ref[off:off + n]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert rel <= 2e-2, (name, rel)
        off += n


def test_denoiser_training_and_gain(capi):
    """Training and what the trained net gains.  With the configuration's targets (depth ray-cast from the
    fused volume of two new-seed rooms) the training loss falls.  With noise-free targets of the same rooms,
    on a held-out room the net's depth is closer to the true depth than the raw depth and than the bilateral
    filter's (RMSE over pixels valid in all three and within the discontinuity threshold; printed)."""
    from voxelhashmt_gb300 import _capi, backend, denoiser, scenes
    raws, tgts = denoiser.make_training_pairs([101, 102], frames_per_scene=40, crops_per_frame=8)
    net = denoiser.DepthDenoiser(seed=1)
    hist = denoiser.train(net, raws, tgts, steps=300, batch=16)
    assert np.mean(hist[-30:]) < 0.97 * np.mean(hist[:5]), (hist[:5], hist[-30:])
    raws, tgts = denoiser.make_training_pairs([101, 102], frames_per_scene=40, crops_per_frame=8, target="clean")
    net = denoiser.DepthDenoiser(seed=1)
    denoiser.train(net, raws, tgts, steps=600, batch=16)
    ev_raw, ev_tgt = denoiser.make_training_pairs([203], frames_per_scene=12, crops_per_frame=4, rng_seed=9,
                                                  target="clean")
    out = net.forward(ev_raw)
    vol = backend.VoxelHashTSDF(0.005, 0.02, max_blocks=1)
    K = scenes.Intrinsics(128, 128, 105.0, 105.0, 63.5, 63.5)
    bil = torch.empty_like(ev_raw)
    for i in range(ev_raw.shape[0]):
        _capi.check(_capi.lib().vh_filter_depth(vol.handle, C.c_void_p(ev_raw[i].data_ptr()),
                                                C.c_void_p(bil[i].data_ptr()), C.byref(_capi.intrinsics(K)), None),
                    vol.handle)
    torch.cuda.synchronize()
    gate = torch.clamp(0.025 * ev_tgt, min=0.012)
    m = (ev_raw > 0) & (ev_tgt > 0) & (out > 0) & (bil > 0) & ((ev_raw - ev_tgt).abs() <= gate)

    def rmse(x):
        return float(torch.sqrt(((x - ev_tgt)[m] ** 2).mean()))

    print("held-out RMSE to the true depth (mm): raw %.3f, bilateral %.3f, learned %.3f"
          % (1000 * rmse(ev_raw), 1000 * rmse(bil), 1000 * rmse(out)))
    assert rmse(out) < rmse(bil) and rmse(out) < rmse(ev_raw)
    vol.close()


def test_conv32_bounded_wait_gives_up_and_context_stays_usable(capi):
    """Failure detection without a GPU fault: a load gate that nothing opens leaves every wait of the tensor-core
    convolution unanswered.  Each gives up after about a second, the error word gets the timeout bit, the output
    is left unwritten, and the next launches on the same context run and match."""
    import time
    B, H, W = 1, 12, 200
    g = torch.Generator().manual_seed(11)
    x = torch.randn(B, H, W, 32, generator=g).to(torch.bfloat16).cuda().contiguous()
    w = (torch.randn(32, 32, 3, 3, generator=g) * 0.1).float().cuda().contiguous()
    b = (torch.randn(32, generator=g) * 0.1).float().cuda().contiguous()
    packed = torch.empty(9 * 32 * 32, dtype=torch.bfloat16, device="cuda")
    capi.check(capi.lib().vh_nn_pack_conv32_weights(_ptr(w), _ptr(packed), 0, None))
    want = _run(capi, x, w, b, None, 0, 1)

    def gated(open_gate):
        gate = torch.full((1,), 1 if open_gate else 0, dtype=torch.int32, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        out = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        capi.check(capi.lib().vh_nn_conv32_gated(_ptr(x), _ptr(packed), _ptr(b), None, _ptr(out), B, W, H, 0, 1,
                                                 _ptr(gate), C.cast(C.c_void_p(err.data_ptr()), C.POINTER(C.c_uint32)),
                                                 None))
        torch.cuda.synchronize()
        return out, int(err.item()), time.perf_counter() - t0

    out, err, secs = gated(False)
    assert err & 8, "the timeout bit was not set"
    assert 0.5 < secs < 30.0, secs
    assert torch.isnan(out.float()).all(), "a timed-out launch wrote output"
    out, err, _ = gated(True)
    assert err == 0 and torch.equal(out, want)
    again = _run(capi, x, w, b, None, 0, 1)  # the ungated kernel after the timeout
    assert torch.equal(again, want)
