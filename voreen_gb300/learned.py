"""The learned upsampler: a 3-level BF16 U-Net (32/64/128 channels, 3x3
convolutions, FP32 accumulation on the tensor cores) that rebuilds the
full-resolution, full-rate frame from a half-resolution, half-rate march.

All arithmetic runs in the library's own kernels (include/vrc_nn.h); torch
only holds device buffers and orders work on its current stream.

Network (input h x w, output 2h x 2w RGBA):
    x0  = [rgba, first-hit depth, |gradient|, 0...]         16 ch   h x w
    e1  = relu(conv(relu(conv(x0, 32)), 32))                       h x w
    e2  = relu(conv(relu(conv(avgpool(e1), 64)), 64))              h/2
    b   = relu(conv(relu(conv(avgpool(e2), 128)), 128))            h/4
    d2  = relu(conv(relu(conv([up(b) | e2], 64)), 64))             h/2
    d1  = relu(conv(relu(conv([up(d2) | e1], 32)), 32))            h
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

LAYERS = [  # name, Cin, Cout, relu
    ("enc1a", 16, 32, 1), ("enc1b", 32, 32, 1),
    ("enc2a", 32, 64, 1), ("enc2b", 64, 64, 1),
    ("bota", 64, 128, 1), ("botb", 128, 128, 1),
    ("dec2a", 192, 64, 1), ("dec2b", 64, 64, 1),
    ("dec1a", 96, 32, 1), ("dec1b", 32, 32, 1),
    ("head", 32, 16, 0),
]

_NN = None


def nn_lib():
    """The library with the vrc_nn_* signatures set."""
    global _NN
    if _NN is None:
        L = _abi.load()
        VP, I, F, LL = C.c_void_p, C.c_int, C.c_float, C.c_longlong
        sig = {
            "vrc_nn_conv3x3_fwd": [VP, I, I, I, I, VP, VP, I, I, VP, I, VP],
            "vrc_nn_conv3x3_wgrad": [VP, VP, I, I, I, I, I, VP, VP, VP],
            "vrc_nn_flip_weights": [VP, I, I, VP, VP],
            "vrc_nn_relu_bwd": [VP, VP, LL, VP],
            "vrc_nn_avgpool2": [VP, I, I, I, I, F, VP, VP],
            "vrc_nn_upsample2": [VP, I, I, I, I, F, VP, VP],
            "vrc_nn_concat": [VP, I, VP, I, LL, VP, I, VP],
            "vrc_nn_add": [VP, VP, LL, VP],
            "vrc_nn_head_fwd": [VP, VP, I, I, I, VP, VP],
            "vrc_nn_head_bwd": [VP, I, I, I, VP, VP],
            "vrc_nn_bilinear_up2": [VP, I, I, I, VP, VP],
            "vrc_nn_loss": [VP, VP, I, I, I, I, F, VP, VP, VP, VP],
            "vrc_nn_adam": [VP, VP, VP, VP, VP, LL, F, F, F, F, I, VP],
            "vrc_nn_pack_input": [VP, VP, LL, VP, VP],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _NN = L
    return _NN


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

    def __init__(self, seed: int = 0, device: str = "cuda"):
        import torch
        self.torch = torch
        self.device = device
        g = torch.Generator().manual_seed(seed)
        self.w, self.b = {}, {}
        for name, cin, cout, _ in LAYERS:
            std = math.sqrt(2.0 / (9 * cin)) if name != "head" else 1e-3
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
        """BF16 copies and the flipped data-gradient weights from the masters."""
        for name, cin, cout, _ in LAYERS:
            self.w16[name].copy_(self.w[name].to(self.torch.bfloat16))
            self.wt16[name] = self.torch.empty((cin, 3, 3, cout), dtype=self.torch.bfloat16, device=self.device)
            _call("vrc_nn_flip_weights", _p(self.w16[name]), cout, cin, _p(self.wt16[name]), _stream())

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
    def forward(self, x0, base):
        """x0: (N, h, w, 16) BF16; base: (N, h, w, 4) FP32 low-res RGBA.
        Returns (N, 2h, 2w, 4) FP32."""
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
        _call("vrc_nn_relu_bwd", _p(y), _p(dy), dy.numel(), _stream())

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
