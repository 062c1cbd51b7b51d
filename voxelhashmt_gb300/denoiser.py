"""Learned depth denoiser that can stand in for the bilateral filter (vh_algorithm.depth_filter = 1).

Net: 3x3 convolutions 4 -> 32 -> 32 -> 32 -> 1 with ReLU, residual output (depth' = depth + r / 100 on valid
pixels).  The input channels per pixel are the depth's local high-pass (centimetres), the validity mask and
the local depth level.  The weights are BF16 in the two 32 -> 32 layers (tensor cores, FP32 accumulation,
BF16 activations); the input and output layers and all weight gradients and Adam moments are FP32.
Every kernel is in the library (vh_nn_*); this module holds the buffers and runs the loop.

Training pairs: raw noisy depth frames and the depth ray-cast (vh_raycast_depth) at the same pose from the
volume fused from all frames of the scene with the plain FP32 pipeline, whole frames or random crops.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def param_count() -> int:
    return int(_capi.lib().vh_nn_param_count())


def init_params(seed=0) -> np.ndarray:
    """He-normal weights, zero biases; the output layer starts small so the net starts near identity."""
    rng = np.random.default_rng(seed)
    parts = []
    for cin, cout, scale in ((4, 32, 1.0), (32, 32, 1.0), (32, 32, 1.0), (32, 1, 0.1)):
        std = scale * np.sqrt(2.0 / (cin * 9))
        parts.append(rng.normal(0.0, std, size=cout * cin * 9))
        parts.append(np.zeros(cout))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == param_count()
    return p


class DepthDenoiser:
    """Parameters, packed tensor-core weights, Adam moments and workspace on one GPU."""

    def __init__(self, params=None, seed=0, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        import torch
        self.torch = torch
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        self.params = torch.from_numpy(p.copy()).cuda()
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.packed = torch.empty(4 * 9 * 32 * 32, dtype=torch.bfloat16, device="cuda")
        self.loss = torch.zeros(2, dtype=torch.float32, device="cuda")
        self.error = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.lr, self.beta1, self.beta2, self.eps = lr, beta1, beta2, eps
        self.step_count = 0
        self._ws = None
        self._ws_shape = None
        self._repack()

    def _err(self):
        return C.cast(C.c_void_p(self.error.data_ptr()), C.POINTER(C.c_uint32))

    def _repack(self):
        _capi.check(_capi.lib().vh_nn_pack(_ptr(self.params), _ptr(self.packed), None))

    def _workspace(self, b, w, h):
        if self._ws_shape != (b, w, h):
            n = int(_capi.lib().vh_nn_workspace_bytes(b, w, h))
            self._ws = self.torch.empty(n, dtype=self.torch.uint8, device="cuda")
            self._ws_shape = (b, w, h)
        return self._ws

    def check_error(self):
        if int(self.error.item()) != 0:
            raise _capi.VhError(_capi.VH_ERR_TIMEOUT, "tensor cores did not signal completion in time")

    def forward(self, depth):
        """depth: (B, H, W) float32 CUDA tensor -> denoised (B, H, W)."""
        depth = depth.contiguous()
        b, h, w = depth.shape
        out = self.torch.empty_like(depth)
        _capi.check(_capi.lib().vh_nn_forward(_ptr(self.params), _ptr(self.packed), _ptr(depth), _ptr(out), b, w, h,
                                              _ptr(self._workspace(b, w, h)), self._err(), None))
        return out

    def train_step(self, raw, target):
        """One Adam step on a batch (B, H, W) of raw depth and targets; returns the batch RMSE (metres) over
        the pixels valid in input, target and output, before the step."""
        raw, target = raw.contiguous(), target.contiguous()
        b, h, w = raw.shape
        out = self.forward(raw)
        ws = self._workspace(b, w, h)
        _capi.check(_capi.lib().vh_nn_backward(_ptr(self.params), _ptr(self.packed), _ptr(raw), _ptr(target), _ptr(out),
                                               b, w, h, _ptr(ws), _ptr(self.grads), _ptr(self.loss), self._err(), None))
        self.step_count += 1
        _capi.check(_capi.lib().vh_nn_adam(_ptr(self.params), _ptr(self.grads), _ptr(self.m), _ptr(self.v), self.lr,
                                           self.beta1, self.beta2, self.eps, self.step_count, None))
        self._repack()
        se, cnt = self.loss.tolist()
        return float(np.sqrt(se / max(cnt, 1.0)))

    def gradients(self, raw, target):
        """(gradients (P,) numpy, loss) of one batch without updating: for checks against a reference."""
        raw, target = raw.contiguous(), target.contiguous()
        b, h, w = raw.shape
        out = self.forward(raw)
        _capi.check(_capi.lib().vh_nn_backward(_ptr(self.params), _ptr(self.packed), _ptr(raw), _ptr(target), _ptr(out),
                                               b, w, h, _ptr(self._workspace(b, w, h)), _ptr(self.grads),
                                               _ptr(self.loss), self._err(), None))
        self.torch.cuda.synchronize()
        self.check_error()
        se = float(self.loss[0].item())
        return self.grads.cpu().numpy(), se / (b * h * w), out

    def params_numpy(self) -> np.ndarray:
        return self.params.cpu().numpy()


def make_training_pairs(seeds, frames_per_scene=120, crops_per_frame=16, crop=128, width=640, height=480,
                        fuse_frames=None, rng_seed=0, target="raycast"):
    """Pairs (raw, target) from rooms (scenes.room_scene) of the given seeds: raw = the noisy rendered frame;
    target = the depth ray-cast at the frame's pose from the plain FP32 volume fused from `fuse_frames` frames
    of the same walk (all of them by default), or with target="clean" the noise-free analytic depth of the
    frame.  crop > 0: random crop x crop windows, crops_per_frame per frame; crop = 0 (or None): whole frames.
    Returns two (N, h, w) CUDA tensors; windows (and frames) are kept where at least half the pixels are valid
    in both."""
    import torch
    from . import backend, scenes
    rng = np.random.default_rng(rng_seed)
    raws, tgts = [], []
    for seed in seeds:
        n_fuse = fuse_frames or frames_per_scene
        sc = scenes.room_scene(seed=seed, frames=max(frames_per_scene, n_fuse), width=width, height=height,
                               fx=525.0 * width / 640, fy=525.0 * width / 640, cx=(width - 1) / 2, cy=(height - 1) / 2)
        frames = render_frames(sc, torch)
        clean = None
        vol = None
        if target == "clean":
            noise, drop = sc.noise_sigma_z2, sc.dropout
            sc.noise_sigma_z2, sc.dropout = 0.0, 0.0
            clean = render_frames(sc, torch)
            sc.noise_sigma_z2, sc.dropout = noise, drop
        else:
            vol = backend.VoxelHashTSDF(sc.voxel_size, sc.truncation, hash_buckets=sc.hash_buckets,
                                        max_blocks=600_000)
            bk = backend.TsdfIntegrationBackend("gpu")
            for f in range(n_fuse):
                bk.integrate(vol, backend.DepthFrame(sc.intrinsics, frames[f].view(-1)), sc.poses[f], 1,
                             synchronize=False)
            vol.synchronize()
        for f in range(frames_per_scene):
            if clean is not None:
                tgt = clean[f]
            else:
                tgt = backend.raycast_depth(vol, sc.intrinsics, sc.poses[f], 0.1, sc.max_depth, 0.5,
                                            device_out="cuda")
            raw = frames[f]
            if not crop:
                if float(((raw > 0) & (tgt > 0)).float().mean()) >= 0.5:
                    raws.append(raw.clone())
                    tgts.append(tgt.clone())
                continue
            taken = 0
            for _ in range(crops_per_frame * 4):  # bounded retries for windows with too little valid depth
                if taken >= crops_per_frame:
                    break
                y0 = int(rng.integers(0, height - crop + 1))
                x0 = int(rng.integers(0, width - crop + 1))
                r = raw[y0:y0 + crop, x0:x0 + crop]
                t = tgt[y0:y0 + crop, x0:x0 + crop]
                if float(((r > 0) & (t > 0)).float().mean()) >= 0.5:
                    raws.append(r.clone())
                    tgts.append(t.clone())
                    taken += 1
        if vol is not None:
            vol.close()
    return torch.stack(raws), torch.stack(tgts)


def render_frames(sc, torch):
    """All frames of a scene rendered on the device (noise as configured in the scene)."""
    prims = torch.from_numpy(np.ascontiguousarray(sc.prims, np.float32)).cuda()
    K = sc.intrinsics
    out = torch.empty((len(sc.poses), K.height, K.width), dtype=torch.float32, device="cuda")
    Kc = _capi.intrinsics(K)
    for f in range(len(sc.poses)):
        P = _capi.pose(sc.poses[f])
        _capi.check(_capi.lib().vh_render_depth(_ptr(prims), prims.shape[0], C.byref(Kc), C.byref(P), sc.seed, f,
                                                sc.noise_sigma_z2, sc.dropout, sc.max_depth, _ptr(out[f]), None))
    torch.cuda.synchronize()
    return out


def train(denoiser: DepthDenoiser, raws, targets, steps, batch=16, seed=0, log_every=0):
    """Adam over random batches of the pairs; returns the per-step RMSE list."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for s in range(steps):
        idx = torch.randint(0, raws.shape[0], (batch,), generator=g).cuda()
        hist.append(denoiser.train_step(raws[idx], targets[idx]))
        if log_every and s % log_every == 0:
            print("step %d rmse %.5f" % (s, hist[-1]), flush=True)
    torch.cuda.synchronize()
    denoiser.check_error()
    return hist


def _time_forward(frames=20, batch=1, seed=3):
    """Forward passes of a seeded net over rendered 640x480 room frames: (ms per pass, batch)."""
    import torch
    from . import build, scenes
    build.build()
    torch.cuda.set_device(0)
    sc = scenes.room_scene(seed=5, frames=4)
    depth = render_frames(sc, torch)
    net = DepthDenoiser(seed=seed)
    x = depth[:1].repeat(batch, 1, 1) if batch > 1 else depth[:1]
    for _ in range(3):
        net.forward(x)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(frames):
        net.forward(x if batch > 1 else depth[i % 4:i % 4 + 1])
    e1.record()
    torch.cuda.synchronize()
    net.check_error()
    return e0.elapsed_time(e1) / frames


def _time_train_step(steps=20, batch=16, seed=1):
    """Adam steps of a seeded net on rendered 640x480 room frames (noise-free targets), after 3 warm-up steps:
    (forward, backward, Adam + weight packing) ms per step, CUDA events."""
    import torch
    from . import build, scenes
    build.build()
    torch.cuda.set_device(0)
    sc = scenes.room_scene(seed=5, frames=batch)
    raw = render_frames(sc, torch)
    sc.noise_sigma_z2, sc.dropout = 0.0, 0.0
    tgt = render_frames(sc, torch)
    net = DepthDenoiser(seed=seed)
    b, h, w = raw.shape
    lib = _capi.lib()
    for _ in range(3):
        net.train_step(raw, tgt)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    tf = tb = ta = 0.0
    for _ in range(steps):
        ev[0].record()
        out = net.forward(raw)
        ev[1].record()
        _capi.check(lib.vh_nn_backward(_ptr(net.params), _ptr(net.packed), _ptr(raw), _ptr(tgt), _ptr(out), b, w, h,
                                       _ptr(net._workspace(b, w, h)), _ptr(net.grads), _ptr(net.loss), net._err(),
                                       None))
        ev[2].record()
        net.step_count += 1
        _capi.check(lib.vh_nn_adam(_ptr(net.params), _ptr(net.grads), _ptr(net.m), _ptr(net.v), net.lr, net.beta1,
                                   net.beta2, net.eps, net.step_count, None))
        net._repack()
        ev[3].record()
        torch.cuda.synchronize()
        tf += ev[0].elapsed_time(ev[1])
        tb += ev[1].elapsed_time(ev[2])
        ta += ev[2].elapsed_time(ev[3])
    net.check_error()
    return tf / steps, tb / steps, ta / steps


if __name__ == "__main__":
    # python -m voxelhashmt_gb300.denoiser [--frames N] [--batch B]: time the net's forward pass;
    # with --train: time training steps (batch B, default 16)
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=20)
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--train", action="store_true")
    a = ap.parse_args()
    if a.train:
        bt = a.batch or 16
        f, bw, ad = _time_train_step(a.frames, bt)
        print("denoiser training step, batch %d x 640x480: forward %.3f ms, backward %.3f ms, Adam + packing %.3f ms"
              % (bt, f, bw, ad))
    else:
        bt = a.batch or 1
        ms = _time_forward(a.frames, bt)
        print("denoiser forward: %.4f ms per pass of %d 640x480 frame(s)" % (ms, bt))
