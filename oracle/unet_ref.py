"""FP64 numpy reference of the learned upsampler -- TEST INFRASTRUCTURE ONLY.

Restates the network of voreen_gb300/learned.py (3x3 convolutions, ReLU,
2x2 average pool, nearest 2x upsample, channel concat, depth-to-space head
plus bilinear residual) and its L1 + SSIM loss, with forward and backward in
float64, so the GPU kernels' activations and gradients can be checked.
Tensors are NHWC; weights [Cout][3][3][Cin].
"""
from __future__ import annotations

import numpy as np

LAYERS = [("enc1a", 16, 32, 2), ("enc1b", 32, 32, 2), ("enc2a", 32, 64, 2), ("enc2b", 64, 64, 2),
          ("bota", 64, 128, 2), ("botb", 128, 128, 2), ("dec2a", 192, 64, 2), ("dec2b", 64, 64, 2),
          ("dec1a", 96, 32, 2), ("dec1b", 32, 32, 2), ("head", 32, 16, 0)]
LEAK = 0.05
C1, C2 = 0.01 ** 2, 0.03 ** 2


def conv3x3(x, w, b=None):
    N, H, W, Ci = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((N, H, W, w.shape[0]))
    for kh in range(3):
        for kw in range(3):
            out += np.einsum("nhwc,oc->nhwo", xp[:, kh:kh + H, kw:kw + W, :], w[:, kh, kw, :], optimize=True)
    if b is not None:
        out += b
    return out


def conv3x3_wgrad(x, dy):
    N, H, W, Ci = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((dy.shape[3], 3, 3, Ci))
    for kh in range(3):
        for kw in range(3):
            dw[:, kh, kw, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, kh:kh + H, kw:kw + W, :], optimize=True)
    return dw, dy.sum(axis=(0, 1, 2))


def conv3x3_dgrad(dy, w):
    wt = np.transpose(w[:, ::-1, ::-1, :], (3, 1, 2, 0))  # [ci][kh][kw][co]
    return conv3x3(dy, wt)


def avgpool(x):
    return 0.25 * (x[:, 0::2, 0::2] + x[:, 1::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 1::2])


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def bilinear_up2(base):
    N, H, W, _ = base.shape
    oy = np.arange(2 * H)
    ox = np.arange(2 * W)
    sy = np.maximum((oy + 0.5) * 0.5 - 0.5, 0)
    sx = np.maximum((ox + 0.5) * 0.5 - 0.5, 0)
    y0 = np.minimum(sy.astype(int), H - 1)
    x0 = np.minimum(sx.astype(int), W - 1)
    y1 = np.minimum(y0 + 1, H - 1)
    x1 = np.minimum(x0 + 1, W - 1)
    fy = (sy - y0)[None, :, None, None]
    fx = (sx - x0)[None, None, :, None]
    g = lambda yy, xx: base[:, yy][:, :, xx]
    return (g(y0, x0) * (1 - fx) + g(y0, x1) * fx) * (1 - fy) + (g(y1, x0) * (1 - fx) + g(y1, x1) * fx) * fy


def depth_to_space(f):
    N, H, W, _ = f.shape
    out = np.zeros((N, 2 * H, 2 * W, 4))
    for dy in range(2):
        for dx in range(2):
            q = 2 * dy + dx
            out[:, dy::2, dx::2, :] = f[:, :, :, 4 * q:4 * q + 4]
    return out


def space_to_depth(d):
    N, H2, W2, _ = d.shape
    f = np.zeros((N, H2 // 2, W2 // 2, 16))
    for dy in range(2):
        for dx in range(2):
            q = 2 * dy + dx
            f[:, :, :, 4 * q:4 * q + 4] = d[:, dy::2, dx::2, :]
    return f


def forward(params, x0, base):
    w, b = params
    a = {"x0": x0}
    r = lambda v: np.where(v > 0, v, LEAK * v)  # leaky ReLU
    a["e1a"] = r(conv3x3(x0, w["enc1a"], b["enc1a"]))
    a["e1"] = r(conv3x3(a["e1a"], w["enc1b"], b["enc1b"]))
    a["p1"] = avgpool(a["e1"])
    a["e2a"] = r(conv3x3(a["p1"], w["enc2a"], b["enc2a"]))
    a["e2"] = r(conv3x3(a["e2a"], w["enc2b"], b["enc2b"]))
    a["p2"] = avgpool(a["e2"])
    a["b1"] = r(conv3x3(a["p2"], w["bota"], b["bota"]))
    a["b2"] = r(conv3x3(a["b1"], w["botb"], b["botb"]))
    a["c2"] = np.concatenate([up(a["b2"]), a["e2"]], axis=3)
    a["d2a"] = r(conv3x3(a["c2"], w["dec2a"], b["dec2a"]))
    a["d2"] = r(conv3x3(a["d2a"], w["dec2b"], b["dec2b"]))
    a["c1"] = np.concatenate([up(a["d2"]), a["e1"]], axis=3)
    a["d1a"] = r(conv3x3(a["c1"], w["dec1a"], b["dec1a"]))
    a["d1"] = r(conv3x3(a["d1a"], w["dec1b"], b["dec1b"]))
    a["f"] = conv3x3(a["d1"], w["head"], b["head"])
    out = depth_to_space(a["f"]) + bilinear_up2(base)
    return out, a


def backward(params, a, dout):
    w, _ = params
    gw, gb = {}, {}
    m = lambda y, d: d * np.where(y > 0, 1.0, LEAK)

    def lay(name, x, dy):
        gw[name], gb[name] = conv3x3_wgrad(x, dy)
        return conv3x3_dgrad(dy, w[name])

    df = space_to_depth(dout)
    dd1 = m(a["d1"], lay("head", a["d1"], df))
    dd1a = m(a["d1a"], lay("dec1b", a["d1a"], dd1))
    dc1 = lay("dec1a", a["c1"], dd1a)
    du1, de1_skip = dc1[..., :64], dc1[..., 64:]
    dd2 = m(a["d2"], 4 * avgpool(du1))
    dd2a = m(a["d2a"], lay("dec2b", a["d2a"], dd2))
    dc2 = lay("dec2a", a["c2"], dd2a)
    du2, de2_skip = dc2[..., :128], dc2[..., 128:]
    db2 = m(a["b2"], 4 * avgpool(du2))
    db1 = m(a["b1"], lay("botb", a["b1"], db2))
    dp2 = lay("bota", a["p2"], db1)
    de2 = m(a["e2"], 0.25 * up(dp2) + de2_skip)
    de2a = m(a["e2a"], lay("enc2b", a["e2a"], de2))
    dp1 = lay("enc2a", a["p1"], de2a)
    de1 = m(a["e1"], 0.25 * up(dp1) + de1_skip)
    de1a = m(a["e1a"], lay("enc1b", a["e1a"], de1))
    lay("enc1a", a["x0"], de1a)
    return gw, gb


def box_stats(img, r):
    N, H, W, Cc = img.shape
    out = np.zeros_like(img)
    cnt = np.zeros((H, W))
    for dy in range(-r, r + 1):
        for dx in range(-r, r + 1):
            ys = slice(max(0, -dy), min(H, H - dy))
            xs = slice(max(0, -dx), min(W, W - dx))
            yd = slice(max(0, dy), min(H, H + dy))
            xd = slice(max(0, dx), min(W, W + dx))
            out[:, ys, xs] += img[:, yd, xd]
            cnt[ys, xs] += 1
    return out, cnt[None, :, :, None]


def loss(x, y, r=2, lam=0.2):
    sx, cnt = box_stats(x, r)
    sy, _ = box_stats(y, r)
    sxx, _ = box_stats(x * x, r)
    syy, _ = box_stats(y * y, r)
    sxy, _ = box_stats(x * y, r)
    mx, my = sx / cnt, sy / cnt
    vx, vy, cxy = sxx / cnt - mx * mx, syy / cnt - my * my, sxy / cnt - mx * my
    S = ((2 * mx * my + C1) * (2 * cxy + C2)) / ((mx * mx + my * my + C1) * (vx + vy + C2))
    return np.abs(x - y).mean() + lam * (1 - S.mean())


def loss_grad_numeric(x, y, idx, r=2, lam=0.2, h=1e-6):
    """Central difference of `loss` w.r.t. x at flat indices idx."""
    g = []
    flat = x.reshape(-1)
    for i in idx:
        old = flat[i]
        flat[i] = old + h
        lp = loss(x, y, r, lam)
        flat[i] = old - h
        lm = loss(x, y, r, lam)
        flat[i] = old
        g.append((lp - lm) / (2 * h))
    return np.array(g)
