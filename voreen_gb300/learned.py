"""The learned upsampler: a 3-level BF16 U-Net (32/64/128 channels, 3x3
convolutions, FP32 accumulation on the tensor cores) that rebuilds the
full-resolution, full-rate frame from a half-resolution, half-rate march.

All arithmetic runs in the library's own kernels (include/vrc_nn.h); torch
only holds device buffers and orders work on its current stream.

Network (input h x w, output 2h x 2w RGBA):
    x0  = [rgba, first-hit depth, |gradient|, 0...]         16 ch   h x w
    e1  = act(conv(act(conv(x0, 32)), 32))   act: leaky ReLU                       h x w
    e2  = act(conv(act(conv(avgpool(e1), 64)), 64))              h/2
    b   = act(conv(act(conv(avgpool(e2), 128)), 128))            h/4
    d2  = act(conv(act(conv([up(b) | e2], 64)), 64))             h/2
    d1  = act(conv(act(conv([up(d2) | e1], 32)), 32))            h
    out = depth_to_space(conv(d1, 16)) + bilinear_up(rgba)         2h x 2w
The last term makes the network learn a residual on the interpolated march.
"""
from __future__ import annotations

import ctypes as C
import io
import json
import math

import numpy as np

from . import _abi

LAYERS = [  # name, Cin, Cout, activation (2: leaky ReLU, 0: none)
    ("enc1a", 16, 32, 2), ("enc1b", 32, 32, 2),
    ("enc2a", 32, 64, 2), ("enc2b", 64, 64, 2),
    ("bota", 64, 128, 2), ("botb", 128, 128, 2),
    ("dec2a", 192, 64, 2), ("dec2b", 64, 64, 2),
    ("dec1a", 96, 32, 2), ("dec1b", 32, 32, 2),
    ("head", 32, 16, 0),
]
LEAK = 0.05
# Inference layers run on the tcgen05 convolution where it is faster than the
# mma.sync one on a GB300 at 960 x 540 (measured per layer, microseconds,
# tcgen05 / mma.sync): enc2a 23 / 25, enc2b 33 / 41, bota 15 / 29, botb 31 / 50,
# dec2b 33 / 41. With 32 or fewer output channels an MMA of N <= 32 costs
# about as much as one of N = 64, so the full-resolution layers (enc1a/b,
# dec1b, head: 40-54 / 25-39) and the decoder inputs [upsample | skip]
# (fused on load by the mma.sync form) stay on mma.sync.
TC_LAYERS = ("enc2a", "enc2b", "bota", "botb", "dec2b")
# Output-channel slices per CTA of the tcgen05 convolution, chosen so each
# slice's weights (9 x Cin x Cout / split BF16) stay in shared memory beside
# the operand stages.
TC_SPLIT = {"botb": 2}

_NN = None


def nn_lib():
    """The library (signatures of include/vrc_nn.h are set by _abi.load)."""
    return _abi.load()


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _call(name, *args):
    st = getattr(nn_lib(), name)(*args)
    if st != 0:
        raise RuntimeError(f"{name} failed with status {st}")


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class UNet:
    """Parameters (FP32 master, BF16 working copies), activations, gradients
    and Adam state of the upsampler, on one CUDA device."""

    def __init__(self, seed: int = 0, device: str = "cuda", head_std: float = 1e-2):
        import torch
        self.torch = torch
        self.device = device
        g = torch.Generator().manual_seed(seed)
        self.w, self.b = {}, {}
        for name, cin, cout, _ in LAYERS:
            std = math.sqrt(2.0 / (9 * cin)) if name != "head" else head_std
            self.w[name] = (torch.randn((cout, 3, 3, cin), generator=g) * std).to(device)
            self.b[name] = torch.zeros(cout, device=device)
        self.step = 0
        self._alloc_state()
        self.refresh()

    # -- parameters -----------------------------------------------------------
    def _alloc_state(self):
        t = self.torch
        self.w16 = {k: v.to(t.bfloat16) for k, v in self.w.items()}
        self.wt16 = {}
        self.gw = {k: t.zeros_like(v) for k, v in self.w.items()}
        self.gb = {k: t.zeros_like(v) for k, v in self.b.items()}
        self.mw = {k: t.zeros_like(v) for k, v in self.w.items()}
        self.vw = {k: t.zeros_like(v) for k, v in self.w.items()}
        self.mb = {k: t.zeros_like(v) for k, v in self.b.items()}
        self.vb = {k: t.zeros_like(v) for k, v in self.b.items()}

    def refresh(self):
        """BF16 copies and the flipped data-gradient weights from the masters
        (the tcgen05 inference weights follow on the next infer_tc)."""
        for name, cin, cout, _ in LAYERS:
            self.w16[name].copy_(self.w[name].to(self.torch.bfloat16))
            self.wt16[name] = self.torch.empty((cin, 3, 3, cout), dtype=self.torch.bfloat16, device=self.device)
            _call("vrc_nn_flip_weights", _p(self.w16[name]), cout, cin, _p(self.wt16[name]), _stream())
        self._wtc_step = None

    def state_dict(self):
        return {"step": self.step, "w": {k: v.cpu().numpy() for k, v in self.w.items()},
                "b": {k: v.cpu().numpy() for k, v in self.b.items()}}

    def save(self, path: str):
        sd = self.state_dict()
        arrays = {f"w.{k}": v for k, v in sd["w"].items()}
        arrays.update({f"b.{k}": v for k, v in sd["b"].items()})
        arrays["step"] = np.array([sd["step"]])
        np.savez(path, **arrays)

    def load(self, path: str):
        z = np.load(path)
        for name, *_ in LAYERS:
            self.w[name].copy_(self.torch.from_numpy(z[f"w.{name}"]))
            self.b[name].copy_(self.torch.from_numpy(z[f"b.{name}"]))
        self.step = int(z["step"][0])
        self.refresh()

    # -- layers ----------------------------------------------------------------
    def _conv(self, name, x, N, H, W, out_f32=False):
        t = self.torch
        _, cin, cout, relu = next(l for l in LAYERS if l[0] == name)
        y = t.empty((N, H, W, cout), dtype=t.float32 if out_f32 else t.bfloat16, device=self.device)
        _call("vrc_nn_conv3x3_fwd", _p(x), N, H, W, cin, _p(self.w16[name]), _p(self.b[name]), cout, relu, _p(y),
              1 if out_f32 else 0, _stream())
        return y

    def _pool(self, x, scale=1.0):
        N, H, W, Cc = x.shape
        y = self.torch.empty((N, H // 2, W // 2, Cc), dtype=self.torch.bfloat16, device=self.device)
        _call("vrc_nn_avgpool2", _p(x), N, H, W, Cc, float(scale), _p(y), _stream())
        return y

    def _up(self, x, scale=1.0):
        N, H, W, Cc = x.shape
        y = self.torch.empty((N, 2 * H, 2 * W, Cc), dtype=self.torch.bfloat16, device=self.device)
        _call("vrc_nn_upsample2", _p(x), N, H, W, Cc, float(scale), _p(y), _stream())
        return y

    def _cat(self, a, b):
        N, H, W, Ca = a.shape
        Cb = b.shape[3]
        y = self.torch.empty((N, H, W, Ca + Cb), dtype=self.torch.bfloat16, device=self.device)
        _call("vrc_nn_concat", _p(a), Ca, _p(b), Cb, N * H * W, _p(y), 0, _stream())
        return y

    # -- forward / backward -----------------------------------------------------
    def _conv_upcat(self, name, a_half, b, N, H, W):
        """Decoder conv reading [up2(a_half) | b] on load (inference)."""
        t = self.torch
        _, cin, cout, relu = next(l for l in LAYERS if l[0] == name)
        y = t.empty((N, H, W, cout), dtype=t.bfloat16, device=self.device)
        _call("vrc_nn_conv3x3_fwd_upcat", _p(a_half), a_half.shape[3], _p(b), b.shape[3], N, H, W,
              _p(self.w16[name]), _p(self.b[name]), cout, relu, _p(y), 0, _stream())
        return y

    # -- inference on the tcgen05 tensor cores ---------------------------------
    def _tbuf(self, key, shape, dtype):
        bufs = self.__dict__.setdefault("_tc_bufs", {})
        b = bufs.get(key)
        if b is None or tuple(b.shape) != tuple(shape) or b.dtype != dtype:
            b = self.torch.empty(shape, dtype=dtype, device=self.device)
            bufs[key] = b
        return b

    def _conv_tc(self, name, x, x1, N, H, W, err, out_f32=False):
        t = self.torch
        _, cin, cout, act = next(l for l in LAYERS if l[0] == name)
        c0 = x.shape[3]
        c1 = x1.shape[3] if x1 is not None else 0
        assert cin == c0 + c1
        y = self._tbuf(name, (N, H, W, cout), t.float32 if out_f32 else t.bfloat16)
        _call("vrc_nn_conv3x3_tc", _p(x), c0, _p(x1) if x1 is not None else None, c1, N, H, W, _p(self.wtc[name]),
              _p(self.b[name]), cout, TC_SPLIT.get(name, 1), act, _p(y), 1 if out_f32 else 0,
              _p(err) if err is not None else None, _stream())
        return y

    def _pool_tc(self, key, x):
        N, H, W, Cc = x.shape
        y = self._tbuf(key, (N, H // 2, W // 2, Cc), self.torch.bfloat16)
        _call("vrc_nn_avgpool2", _p(x), N, H, W, Cc, 1.0, _p(y), _stream())
        return y

    def infer_tc(self, x0, base, out=None, err=None):
        """infer() with the layers of TC_LAYERS on the tcgen05 convolution:
        x0 (N, h, w, 16) BF16 NHWC (h, w multiples of 4), base (N, h, w, 4)
        FP32. err: optional 4-byte device word the tcgen05 convolutions set
        when a bounded wait gives up."""
        t = self.torch
        if getattr(self, "_wtc_step", None) != self.step:  # weights changed since the last rearrangement
            self.wtc = {}
            for name, cin, cout, _ in LAYERS:
                if name in TC_LAYERS:
                    self.wtc[name] = t.empty_like(self.w16[name])
                    _call("vrc_nn_weights_tc", _p(self.w16[name]), cout, cin, 0, TC_SPLIT.get(name, 1),
                          _p(self.wtc[name]), _stream())
            self._wtc_step = self.step

        def conv(name, x, N, H, W, out_f32=False):
            if name in TC_LAYERS:
                return self._conv_tc(name, x, None, N, H, W, err, out_f32)
            return self._conv(name, x, N, H, W, out_f32)

        N, H, W, _ = x0.shape
        H2, W2, H4, W4 = H // 2, W // 2, H // 4, W // 4
        e1 = conv("enc1b", conv("enc1a", x0, N, H, W), N, H, W)
        e2 = conv("enc2b", conv("enc2a", self._pool_tc("p1", e1), N, H2, W2), N, H2, W2)
        b2 = conv("botb", conv("bota", self._pool_tc("p2", e2), N, H4, W4), N, H4, W4)
        d2 = conv("dec2b", self._conv_upcat("dec2a", b2, e2, N, H2, W2), N, H2, W2)
        d1 = conv("dec1b", self._conv_upcat("dec1a", d2, e1, N, H, W), N, H, W)
        f = conv("head", d1, N, H, W, out_f32=True)
        if out is None:
            out = t.empty((N, 2 * H, 2 * W, 4), dtype=t.float32, device=self.device)
        _call("vrc_nn_head_fwd", _p(f), _p(base), N, H, W, _p(out), _stream())
        return out

    def infer(self, x0, base, out=None):
        """Forward without keeping activations; the decoder convolutions build
        [upsample | skip] on load. Same values as forward()."""
        t = self.torch
        N, H, W, _ = x0.shape
        e1 = self._conv("enc1b", self._conv("enc1a", x0, N, H, W), N, H, W)
        e2 = self._conv("enc2b", self._conv("enc2a", self._pool(e1), N, H // 2, W // 2), N, H // 2, W // 2)
        b2 = self._conv("botb", self._conv("bota", self._pool(e2), N, H // 4, W // 4), N, H // 4, W // 4)
        d2 = self._conv("dec2b", self._conv_upcat("dec2a", b2, e2, N, H // 2, W // 2), N, H // 2, W // 2)
        d1 = self._conv("dec1b", self._conv_upcat("dec1a", d2, e1, N, H, W), N, H, W)
        f = self._conv("head", d1, N, H, W, out_f32=True)
        if out is None:
            out = t.empty((N, 2 * H, 2 * W, 4), dtype=t.float32, device=self.device)
        _call("vrc_nn_head_fwd", _p(f), _p(base), N, H, W, _p(out), _stream())
        return out

    def forward(self, x0, base):
        """x0: (N, h, w, 16) BF16; base: (N, h, w, 4) FP32 low-res RGBA.
        Returns (N, 2h, 2w, 4) FP32. Keeps the activations for backward()."""
        t = self.torch
        N, H, W, _ = x0.shape
        a = {"x0": x0, "base": base}
        a["e1a"] = self._conv("enc1a", x0, N, H, W)
        a["e1"] = self._conv("enc1b", a["e1a"], N, H, W)
        a["p1"] = self._pool(a["e1"])
        a["e2a"] = self._conv("enc2a", a["p1"], N, H // 2, W // 2)
        a["e2"] = self._conv("enc2b", a["e2a"], N, H // 2, W // 2)
        a["p2"] = self._pool(a["e2"])
        a["b1"] = self._conv("bota", a["p2"], N, H // 4, W // 4)
        a["b2"] = self._conv("botb", a["b1"], N, H // 4, W // 4)
        a["c2"] = self._cat(self._up(a["b2"]), a["e2"])
        a["d2a"] = self._conv("dec2a", a["c2"], N, H // 2, W // 2)
        a["d2"] = self._conv("dec2b", a["d2a"], N, H // 2, W // 2)
        a["c1"] = self._cat(self._up(a["d2"]), a["e1"])
        a["d1a"] = self._conv("dec1a", a["c1"], N, H, W)
        a["d1"] = self._conv("dec1b", a["d1a"], N, H, W)
        a["f"] = self._conv("head", a["d1"], N, H, W, out_f32=True)
        out = t.empty((N, 2 * H, 2 * W, 4), dtype=t.float32, device=self.device)
        _call("vrc_nn_head_fwd", _p(a["f"]), _p(base), N, H, W, _p(out), _stream())
        self.acts = a
        return out

    def _dgrad(self, name, dy, N, H, W, rows=None):
        """dx = conv(dy, flipped weights) for the input channels `rows`."""
        t = self.torch
        _, cin, cout, _ = next(l for l in LAYERS if l[0] == name)
        wt = self.wt16[name] if rows is None else self.wt16[name][rows[0]:rows[1]].contiguous()
        c = cin if rows is None else rows[1] - rows[0]
        dx = t.empty((N, H, W, c), dtype=t.bfloat16, device=self.device)
        _call("vrc_nn_conv3x3_fwd", _p(dy), N, H, W, cout, _p(wt), None, c, 0, _p(dx), 0, _stream())
        return dx

    def _wgrad(self, name, x, dy, N, H, W):
        _, cin, cout, _ = next(l for l in LAYERS if l[0] == name)
        _call("vrc_nn_conv3x3_wgrad", _p(x), _p(dy), N, H, W, cin, cout, _p(self.gw[name]), _p(self.gb[name]),
              _stream())

    def _relu_bwd(self, y, dy):
        _call("vrc_nn_relu_bwd", _p(y), _p(dy), dy.numel(), 1, _stream())

    def backward(self, dout):
        """dout: dL/d(output) (N, 2h, 2w, 4) FP32. Accumulates into gw, gb."""
        t = self.torch
        a = self.acts
        N, H, W, _ = a["x0"].shape
        df = t.empty((N, H, W, 16), dtype=t.bfloat16, device=self.device)
        _call("vrc_nn_head_bwd", _p(dout), N, H, W, _p(df), _stream())
        self._wgrad("head", a["d1"], df, N, H, W)
        dd1 = self._dgrad("head", df, N, H, W)
        self._relu_bwd(a["d1"], dd1)
        self._wgrad("dec1b", a["d1a"], dd1, N, H, W)
        dd1a = self._dgrad("dec1b", dd1, N, H, W)
        self._relu_bwd(a["d1a"], dd1a)
        self._wgrad("dec1a", a["c1"], dd1a, N, H, W)
        du1 = self._dgrad("dec1a", dd1a, N, H, W, rows=(0, 64))
        de1_skip = self._dgrad("dec1a", dd1a, N, H, W, rows=(64, 96))
        dd2 = self._pool(du1, scale=4.0)
        h2, w2 = H // 2, W // 2
        self._relu_bwd(a["d2"], dd2)
        self._wgrad("dec2b", a["d2a"], dd2, N, h2, w2)
        dd2a = self._dgrad("dec2b", dd2, N, h2, w2)
        self._relu_bwd(a["d2a"], dd2a)
        self._wgrad("dec2a", a["c2"], dd2a, N, h2, w2)
        du2 = self._dgrad("dec2a", dd2a, N, h2, w2, rows=(0, 128))
        de2_skip = self._dgrad("dec2a", dd2a, N, h2, w2, rows=(128, 192))
        db2 = self._pool(du2, scale=4.0)
        h4, w4 = H // 4, W // 4
        self._relu_bwd(a["b2"], db2)
        self._wgrad("botb", a["b1"], db2, N, h4, w4)
        db1 = self._dgrad("botb", db2, N, h4, w4)
        self._relu_bwd(a["b1"], db1)
        self._wgrad("bota", a["p2"], db1, N, h4, w4)
        dp2 = self._dgrad("bota", db1, N, h4, w4)
        de2 = self._up(dp2, scale=0.25)
        _call("vrc_nn_add", _p(de2), _p(de2_skip), de2.numel(), _stream())
        self._relu_bwd(a["e2"], de2)
        self._wgrad("enc2b", a["e2a"], de2, N, h2, w2)
        de2a = self._dgrad("enc2b", de2, N, h2, w2)
        self._relu_bwd(a["e2a"], de2a)
        self._wgrad("enc2a", a["p1"], de2a, N, h2, w2)
        dp1 = self._dgrad("enc2a", de2a, N, h2, w2)
        de1 = self._up(dp1, scale=0.25)
        _call("vrc_nn_add", _p(de1), _p(de1_skip), de1.numel(), _stream())
        self._relu_bwd(a["e1"], de1)
        self._wgrad("enc1b", a["e1a"], de1, N, H, W)
        de1a = self._dgrad("enc1b", de1, N, H, W)
        self._relu_bwd(a["e1a"], de1a)
        self._wgrad("enc1a", a["x0"], de1a, N, H, W)

    def zero_grad(self):
        for k in self.gw:
            self.gw[k].zero_()
            self.gb[k].zero_()

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        s = _stream()
        for name, *_ in LAYERS:
            _call("vrc_nn_adam", _p(self.w[name]), _p(self.gw[name]), _p(self.mw[name]), _p(self.vw[name]),
                  _p(self.w16[name]), self.w[name].numel(), lr, b1, b2, eps, self.step, s)
            _call("vrc_nn_adam", _p(self.b[name]), _p(self.gb[name]), _p(self.mb[name]), _p(self.vb[name]), None,
                  self.b[name].numel(), lr, b1, b2, eps, self.step, s)
        for name, cin, cout, _ in LAYERS:
            _call("vrc_nn_flip_weights", _p(self.w16[name]), cout, cin, _p(self.wt16[name]), s)


def loss_and_grad(out, target, radius: int = 2, lam: float = 0.2):
    """L1 + lam * (1 - SSIM) (box windows of (2r+1)^2) and its gradient."""
    import torch
    N, H, W, _ = out.shape
    coef = torch.empty((N, H, W, 4, 3), dtype=torch.float32, device=out.device)
    dx = torch.empty_like(out)
    acc = torch.zeros(2, dtype=torch.float32, device=out.device)
    _call("vrc_nn_loss", _p(out), _p(target), N, H, W, radius, float(lam), _p(coef), _p(dx), _p(acc), _stream())
    n = out.numel()
    l1 = acc[0] / n
    ssim = acc[1] / n
    return l1 + lam * (1 - ssim), dx, (l1, ssim)


def pack_input(rgba, aux2=None):
    """(N, h, w, 4) FP32 [+ (N, h, w, 2) FP32] -> (N, h, w, 16) BF16."""
    import torch
    N, H, W, _ = rgba.shape
    out = torch.empty((N, H, W, 16), dtype=torch.bfloat16, device=rgba.device)
    _call("vrc_nn_pack_input", _p(rgba.contiguous()), _p(aux2.contiguous() if aux2 is not None else None), N * H * W,
          _p(out), _stream())
    return out


def bilinear_up2(rgba):
    import torch
    N, H, W, _ = rgba.shape
    out = torch.empty((N, 2 * H, 2 * W, 4), dtype=torch.float32, device=rgba.device)
    _call("vrc_nn_bilinear_up2", _p(rgba.contiguous()), N, H, W, _p(out), _stream())
    return out


# ---- the learned render path ------------------------------------------------
def low_params(params, factor: int = 2):
    """Half resolution, half sampling rate, analytic entry/exit."""
    from . import EE_ANALYTIC, RenderParams
    q = RenderParams()
    C.memmove(C.byref(q), C.byref(params), C.sizeof(RenderParams))
    q.width, q.height = params.width // factor, params.height // factor
    q.sampling_rate = params.sampling_rate / factor
    q.entry_exit_mode = EE_ANALYTIC
    q.region[:] = [0, 0, 0, 0]
    return q


def march_aux(ctx, vol, tf, params):
    """Plain march into device buffers plus the auxiliary image: returns
    (rgba (1, h, w, 4) FP32, aux (1, h, w, 2) FP32, stats)."""
    import torch
    from . import OUT_RGBA32F, RenderStats, _check, lib
    rgba = torch.empty((1, params.height, params.width, 4), dtype=torch.float32, device="cuda")
    aux = torch.empty((1, params.height, params.width, 2), dtype=torch.float32, device="cuda")
    st = RenderStats()
    torch.cuda.current_stream().synchronize()
    _check(lib().vrc_render_aux(ctx.handle, vol.handle, tf.handle, C.byref(params), None, None, _p(rgba),
                                OUT_RGBA32F, _p(aux), C.byref(st)), ctx, "vrc_render_aux")
    return rgba, aux, st


def plain_frame(ctx, vol, tf, params, region=None):
    """Full plain render (analytic entry/exit) into a device FP32 image."""
    import torch
    from . import EE_ANALYTIC, OUT_RGBA32F, render
    q = low_params(params, 1)
    q.entry_exit_mode = EE_ANALYTIC
    if region is not None:
        q.region[:] = list(region)
    out = torch.zeros((params.height, params.width, 4), dtype=torch.float32, device="cuda")
    torch.cuda.current_stream().synchronize()
    _, st = render(ctx, vol, tf, q, None, None, OUT_RGBA32F, out)
    return out, st


def psnr(a, b):
    """PSNR (peak 1) over all RGBA channels of two images clamped to [0, 1]."""
    import torch
    mse = torch.mean((a.clamp(0, 1) - b.clamp(0, 1)) ** 2).item()
    return float("inf") if mse == 0 else 10.0 * math.log10(1.0 / mse)


class LearnedRenderer:
    """Half-resolution, half-rate march -> U-Net -> full frame, with a probe:
    a probe x probe tile with content (picked from the previous frame's
    low-resolution alpha) of the plain full-rate render is compared with the
    network's frame every call; the frame PSNR is estimated as the tile's
    error spread over the frame's content tiles, and below `psnr_bound` the
    frame is rendered by the plain kernel instead (the fallback). The network
    runs on the tcgen05 convolutions (tensor_cores=True) or the mma.sync ones.
    The probe tile renders on a side stream through vrc_render_noalloc, in
    parallel with the low-resolution march and the network (so a caller must
    not run vrc_render_noalloc concurrently with render()); everything else
    runs on the context's stream, and the only host synchronisation per frame
    reads the probe's error words and the content map."""

    def __init__(self, ctx, net: UNet, probe: int = 64, psnr_bound: float = 40.0, tensor_cores: bool = True):
        import torch
        self.ctx, self.net, self.probe, self.bound = ctx, net, probe, psnr_bound
        self.tensor_cores = tensor_cores
        self.stream = torch.cuda.ExternalStream(ctx.stream)
        # [probe squared error, probe max |d|, convolution timeout word, unused]
        self.err = torch.zeros(4, dtype=torch.float32, device="cuda")
        self.frames = 0
        self.fallbacks = 0
        self._bufs = {}
        self._scores = None   # per probe-tile mean alpha of the previous frame (host)
        self._side = None     # stream of the probe tile
        self._no_side = {}    # volume handle -> the probe tile renders on the context stream
        self._graphs = {}     # (h, w, tensor cores, weights step) -> captured network
        self.use_graphs = True

    def _buf(self, key, shape, dtype):
        import torch
        b = self._bufs.get(key)
        if b is None or tuple(b.shape) != tuple(shape) or b.dtype != dtype:
            b = torch.empty(shape, dtype=dtype, device="cuda")
            self._bufs[key] = b
        return b

    def probe_window(self, W, H):
        """The probe tile: one with content (mean alpha > 0.02 in the previous
        frame's low-resolution march), a different one each frame; without
        that map, a walk over a coarse grid. Returns (x, y, w, h, content
        fraction of the frame or None)."""
        p = self.probe
        nx, ny = max(1, W // p), max(1, H // p)
        if self._scores is not None and self._scores.shape == (ny, nx):
            idx = np.flatnonzero(self._scores.reshape(-1) > 0.02)
            if len(idx):
                k = int(idx[(self.frames * 7919) % len(idx)])
                return (k % nx) * p, (k // nx) * p, min(p, W), min(p, H), len(idx) / (nx * ny)
        k = (self.frames * 7919) % (nx * ny)
        return (k % nx) * p, (k // nx) * p, min(p, W), min(p, H), None

    def _render_plain(self, vol, tf, params, out, region=None):
        from . import EE_ANALYTIC, OUT_RGBA32F, _check, lib
        q = low_params(params, 1)
        q.entry_exit_mode = EE_ANALYTIC
        if region is not None:
            q.region[:] = list(region)
        _check(lib().vrc_render(self.ctx.handle, vol.handle, tf.handle, C.byref(q), None, None, 0, _p(out),
                                OUT_RGBA32F, 1, None), self.ctx, "vrc_render")

    def _start_probe(self, vol, tf, params, ref, region):
        """The probe tile of the plain render, started on a side stream so
        that it runs beside the low-resolution march and the network (it needs
        only the volume, the TF and the window, known before the frame).
        vrc_render_noalloc takes the stream explicitly and renders the same
        pixels as vrc_render; pre-integrated classification, which it does not
        take, and volumes with more empty-space cells than its fixed scratch
        holds (VRC_ERR_SCRATCH_LIMIT) render the tile on the context stream
        instead. Returns the event the frame waits for, or None."""
        import torch
        from . import CLASSIFY_TF, EE_ANALYTIC, OUT_RGBA32F, VrcError, render_noalloc
        if params.classification != CLASSIFY_TF or self._no_side.get(vol.handle.value):
            return None
        q = low_params(params, 1)
        q.entry_exit_mode = EE_ANALYTIC
        q.region[:] = list(region)
        if self._side is None:
            self._side = torch.cuda.Stream()
        # the side stream must not start before the work already queued on
        # the context stream that produced the volume and TF
        self._side.wait_stream(self.stream)
        try:
            render_noalloc(vol, tf, q, None, None, ref, OUT_RGBA32F, self._side.cuda_stream)
        except VrcError as e:
            if _abi.STATUS_NAMES.get(e.status) != "VRC_ERR_SCRATCH_LIMIT":
                raise
            self._no_side[vol.handle.value] = True
            return None
        ev = torch.cuda.Event()
        ev.record(self._side)
        return ev

    def _network(self, x0, rgba, out, lp):
        """The U-Net on fixed buffers. The first frame of a size runs it
        eagerly (which also lays the tcgen05 weights out), the second
        captures its ~15 launches in a CUDA graph, later frames replay it on
        the context stream. Capture failure falls back to eager launches."""
        import torch
        tc = self.tensor_cores and lp.height % 4 == 0 and lp.width % 4 == 0

        def run():
            if tc:
                self.net.infer_tc(x0, rgba, out, err=self.err[2:3])
            else:
                self.net.infer(x0, rgba, out)

        key = (lp.height, lp.width, tc, self.net.step)
        g = self._graphs.get(key)
        if g == "eager" or not self.use_graphs:
            run()
        elif g is None:
            run()
            self._graphs[key] = "warm"
        elif g == "warm":
            graph = torch.cuda.CUDAGraph()
            try:
                torch.cuda.current_stream().synchronize()
                with torch.cuda.graph(graph):
                    run()
                self._graphs[key] = graph
            except RuntimeError:
                self._graphs[key] = "eager"
            if self._graphs[key] == "eager":
                run()
            else:
                graph.replay()
        else:
            g.replay()

    def render(self, vol, tf, params):
        """Returns (frame (H, W, 4) FP32 device tensor, info dict)."""
        import torch
        from . import OUT_RGBA32F, _check, lib
        lp = low_params(params, 2)
        H, W = params.height, params.width
        x, y, w, h, content = self.probe_window(W, H)
        ref = self._buf("probe", (H, W, 4), torch.float32)
        probe_done = self._start_probe(vol, tf, params, ref, (x, y, w, h))
        with torch.cuda.stream(self.stream):
            rgba = self._buf("rgba", (1, lp.height, lp.width, 4), torch.float32)
            aux = self._buf("aux", (1, lp.height, lp.width, 2), torch.float32)
            _check(lib().vrc_render_aux(self.ctx.handle, vol.handle, tf.handle, C.byref(lp), None, None,
                                        _p(rgba), OUT_RGBA32F, _p(aux), None), self.ctx, "vrc_render_aux")
            out = self._buf("out", (1, H, W, 4), torch.float32)
            self.err.zero_()
            x0 = self._buf("x0", (1, lp.height, lp.width, 16), torch.bfloat16)
            _call("vrc_nn_pack_input", _p(rgba), _p(aux), lp.height * lp.width, _p(x0), _stream())
            self._network(x0, rgba, out, lp)
            # content map of this frame (for the next frame's probe), read back with the error words
            ny, nx = max(1, H // self.probe), max(1, W // self.probe)
            scores = self._buf("scores", (ny, nx), torch.float32)
            _call("vrc_nn_tile_alpha", _p(rgba), lp.height, lp.width, self.probe // 2, ny, nx, _p(scores), _stream())
            if probe_done is None:
                self._render_plain(vol, tf, params, ref, region=(x, y, w, h))
            else:
                self.stream.wait_event(probe_done)
            _call("vrc_nn_probe_error", _p(out), _p(ref), W, x, y, w, h, _p(self.err), _stream())
            host = torch.cat([self.err, scores.reshape(-1)]).cpu()  # the one synchronisation
            se, mx = float(host[0]), float(host[1])
            tc_err = int(host[2:3].view(torch.int32)[0])
            if tc_err:
                raise RuntimeError(f"tcgen05 convolution gave up waiting (code {tc_err})")
            self._scores = host[4:].numpy().reshape(ny, nx)
            mse = se / (w * h * 4)
            probe_psnr = float("inf") if mse == 0 else 10 * math.log10(1.0 / mse)
            # frame estimate: the content tile's error spread over the frame's content
            est = mse * content if content is not None else mse
            frame_psnr = float("inf") if est == 0 else 10 * math.log10(1.0 / est)
            self.frames += 1
            fallback = frame_psnr < self.bound
            frame = out[0]
            if fallback:
                self.fallbacks += 1
                frame = self._buf("fallback", (H, W, 4), torch.float32)
                self._render_plain(vol, tf, params, frame)
        return frame, {"probe_psnr": probe_psnr, "frame_psnr_estimate": frame_psnr, "probe_max_abs": mx,
                       "fallback": fallback, "probe": (x, y, w, h)}

    def stage_times(self, vol, tf, params, steps: int = 20):
        """Device milliseconds per frame of each stage of render(), each timed
        alone on the context stream with CUDA events over `steps` repetitions
        (after one untimed run): the half-resolution half-rate march, the
        input packing, the network, the probe tile, and the plain full frame
        a fallback adds. Call after render() has run at this size,
        so that the network is captured."""
        import torch
        from . import OUT_RGBA32F, _check, lib
        lp = low_params(params, 2)
        H, W = params.height, params.width
        rgba = self._buf("rgba", (1, lp.height, lp.width, 4), torch.float32)
        aux = self._buf("aux", (1, lp.height, lp.width, 2), torch.float32)
        x0 = self._buf("x0", (1, lp.height, lp.width, 16), torch.bfloat16)
        out = self._buf("out", (1, H, W, 4), torch.float32)
        ref = self._buf("probe", (H, W, 4), torch.float32)
        full = self._buf("fallback", (H, W, 4), torch.float32)
        x, y, w, h, _ = self.probe_window(W, H)

        def march():
            _check(lib().vrc_render_aux(self.ctx.handle, vol.handle, tf.handle, C.byref(lp), None, None, _p(rgba),
                                        OUT_RGBA32F, _p(aux), None), self.ctx, "vrc_render_aux")

        stages = {
            "march_half": march,
            "pack_input": lambda: _call("vrc_nn_pack_input", _p(rgba), _p(aux), lp.height * lp.width, _p(x0),
                                        _stream()),
            "network": lambda: self._network(x0, rgba, out, lp),
            "probe_tile": lambda: self._render_plain(vol, tf, params, ref, region=(x, y, w, h)),
            "plain_frame": lambda: self._render_plain(vol, tf, params, full),
        }
        res = {}
        with torch.cuda.stream(self.stream):
            for name, fn in stages.items():
                fn()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(self.stream)
                for _ in range(steps):
                    fn()
                b.record(self.stream)
                b.synchronize()
                res[name] = a.elapsed_time(b) / steps
        return res


# ---- training on pairs the plain raycaster renders ---------------------------
def random_view(rng, vox, spacing, seed, width=1920, height=1080):
    """A random orbit camera and a random 5-trapezoid TF on the shell intensities."""
    from . import synth
    dims = (vox.shape[2], vox.shape[1], vox.shape[0])
    keys, domain = synth.shells_tf(vox, seed)
    pos, focus, near, far = synth.orbit_camera(dims, spacing, rng.uniform(0, 360), rng.uniform(-60, 60),
                                               rng.uniform(1.1, 1.8))
    w = synth.Workload("train", vox, spacing, keys, 4096, domain, width, height, 2.0, compositing=0, shading=1,
                       camera_pos=pos, camera_focus=focus, near=near, far=far, light_pos=(*pos, 1.0))
    return w


def random_view_tubes(rng, meta, spacing, seed, width=1920, height=1080):
    """A random orbit camera (closer than the CT family's: tubes are thin) and
    a random 2-peak TF on the tube intensities of a sparse tube volume;
    meta = {"dims": (X, Y, Z), "minmax": (lo, hi)} of the uploaded volume.
    Rate 1.5, Phong, light at the camera, as the large tube workload."""
    from . import synth
    keys, domain = synth.tubes_tf(seed, 2, meta["minmax"])
    pos, focus, near, far = synth.orbit_camera(meta["dims"], spacing, rng.uniform(0, 360), rng.uniform(-60, 60),
                                               rng.uniform(0.9, 1.5))
    return synth.Workload("train tubes", None, spacing, keys, 4096, domain, width, height, 1.5, compositing=0,
                          shading=1, camera_pos=pos, camera_focus=focus, near=near, far=far, light_pos=(*pos, 1.0))


def make_pair(ctx, vol, tf, params):
    """(x0 BF16 (1,h,w,16), low rgba (1,h,w,4), target (1,H,W,4)) for one view."""
    lp = low_params(params, 2)
    rgba, aux, _ = march_aux(ctx, vol, tf, lp)
    target, _ = plain_frame(ctx, vol, tf, params)
    return pack_input(rgba, aux), rgba, target[None]


def crops(x0, base, target, n, size, rng, min_alpha: float = 0.02, tries: int = 8):
    """n random aligned crops (low size x size, high 2size x 2size), each
    re-drawn up to `tries` times until the target's mean alpha exceeds
    `min_alpha` (empty background teaches nothing)."""
    import torch
    _, h, w, _ = x0.shape
    amap = target[0, ..., 3]
    xs, bs, ts = [], [], []
    for _ in range(n):
        for _t in range(tries):
            y = int(rng.integers(0, max(1, h - size + 1)))
            x = int(rng.integers(0, max(1, w - size + 1)))
            if float(amap[2 * y:2 * y + 2 * size, 2 * x:2 * x + 2 * size].mean()) > min_alpha:
                break
        xs.append(x0[:, y:y + size, x:x + size])
        bs.append(base[:, y:y + size, x:x + size])
        ts.append(target[:, 2 * y:2 * y + 2 * size, 2 * x:2 * x + 2 * size])
    return (torch.cat(xs).contiguous(), torch.cat(bs).contiguous(), torch.cat(ts).contiguous())


def train(ctx, net: UNet, volumes, steps: int, seed: int = 0, batch: int = 8, crop: int = 96, lr: float = 2e-4,
          refresh_every: int = 2, log=None, width=1920, height=1080, warmup: int = 200, view_fn=None):
    """Adam on L1 + SSIM over random crops of pairs rendered on the fly from
    `volumes` [(Volume, voxels or meta, spacing)] with random cameras and TFs
    (view_fn: random_view, the CT family, or random_view_tubes)."""
    import random
    import time

    import numpy as np

    from . import TransferFunction
    rng = np.random.default_rng(seed)
    prng = random.Random(seed)
    hist = []
    pair = None
    t0 = time.time()
    for it in range(steps):
        if pair is None or it % refresh_every == 0:
            vol, vox, sp = volumes[int(rng.integers(0, len(volumes)))]
            w = (view_fn or random_view)(prng, vox, sp, int(rng.integers(0, 1 << 30)), width, height)
            tf = TransferFunction(ctx, TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
            pair = make_pair(ctx, vol, tf, w.params())
            tf.close()
        x0, base, target = crops(*pair, batch, crop, rng)
        out = net.forward(x0, base)
        L, dx, (l1, ss) = loss_and_grad(out, target)
        net.zero_grad()
        net.backward(dx)
        cur_lr = lr * min(1.0, (it + 1) / max(1, warmup)) * 0.5 * (1 + math.cos(math.pi * it / max(1, steps)))
        net.adam(lr=cur_lr)
        if log is not None and (it % 100 == 0 or it == steps - 1):
            rec = {"step": it, "loss": float(L), "l1": float(l1), "ssim": float(ss), "lr": cur_lr,
                   "seconds": time.time() - t0}
            hist.append(rec)
            log(rec)
    return hist


def evaluate(ctx, net, volumes, views: int, seed: int, width=1920, height=1080, view_fn=None):
    """PSNR of the learned frame and of the bilinear upsample of the same
    half-resolution march (the method without the network) against the plain
    full render, on `views` random views of `volumes`."""
    import random

    import numpy as np

    from . import TransferFunction
    prng = random.Random(seed)
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(views):
        vol, vox, sp = volumes[int(rng.integers(0, len(volumes)))]
        w = (view_fn or random_view)(prng, vox, sp, int(rng.integers(0, 1 << 30)), width, height)
        tf = TransferFunction(ctx, TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
        x0, base, target = make_pair(ctx, vol, tf, w.params())
        y = net.forward(x0, base)
        bl = bilinear_up2(base)
        out.append({"psnr_net": psnr(y, target), "psnr_bilinear": psnr(bl, target),
                    "max_abs_net": float((y.clamp(0, 1) - target.clamp(0, 1)).abs().max())})
        tf.close()
    return out


def _main():
    import argparse
    import json
    import time

    import torch

    from . import Context, Volume, build, synth, synth_tubes_device, synth_volume
    ap = argparse.ArgumentParser(description="train / evaluate the learned upsampler")
    ap.add_argument("--family", default="ct", choices=["ct", "tubes"],
                    help="ct: 512^3 u16 nested shells (spacing 0.7/0.7/1); tubes: 1024x1024x512 u16 with 125 "
                         "sparse tubes (the large tube workload's density at an eighth of its voxels)")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--train-volumes", type=int, default=4)
    ap.add_argument("--eval-views", type=int, default=8)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--crop", type=int, default=96)
    ap.add_argument("--lr", type=float, default=2e-4)
    ap.add_argument("--head-std", type=float, default=1e-2)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--out", default="upsampler.npz")
    ap.add_argument("--init", default=None)
    args = ap.parse_args()
    build.build()
    ctx = Context(0)
    d = (args.size,) * 3

    def vols(seeds):
        res = []
        for s in seeds:
            if args.family == "tubes":
                dims = (1024, 1024, 512)
                vox = synth_tubes_device(dims, 125, 6000 + s)
                vol = Volume(ctx, vox, (1.0, 1.0, 1.0))
                res.append((vol, {"dims": dims, "minmax": vol.minmax()}, (1.0, 1.0, 1.0)))
            else:
                vox = synth_volume(synth.SHELLS, 1, d, 4000 + s)
                res.append((Volume(ctx, vox, (0.7, 0.7, 1.0)), vox, (0.7, 0.7, 1.0)))
        return res

    view_fn = random_view_tubes if args.family == "tubes" else random_view

    t0 = time.time()
    train_vols = vols(range(args.train_volumes))
    held_out = vols([100, 101])
    net = UNet(seed=0, head_std=args.head_std)
    if args.init:
        net.load(args.init)
    print(json.dumps({"volumes_ready_s": time.time() - t0}), flush=True)
    hist = train(ctx, net, train_vols, args.steps, seed=1, batch=args.batch, crop=args.crop, lr=args.lr,
                 log=lambda r: print(json.dumps(r), flush=True), width=args.width, height=args.height,
                 warmup=args.warmup, view_fn=view_fn)
    torch.cuda.synchronize()
    net.save(args.out)
    ev = evaluate(ctx, net, held_out, args.eval_views, seed=777, width=args.width, height=args.height,
                  view_fn=view_fn)
    print(json.dumps({"eval": ev, "mean_psnr_net": sum(e["psnr_net"] for e in ev) / len(ev),
                      "mean_psnr_bilinear": sum(e["psnr_bilinear"] for e in ev) / len(ev),
                      "train_seconds": hist[-1]["seconds"] if hist else 0}), flush=True)


if __name__ == "__main__":
    _main()
