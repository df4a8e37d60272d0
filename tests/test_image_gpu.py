"""Interaction coarseness: the bilinear rescale of a coarse render to the
output size (VolumeRaycaster::rescaleRendering, GL_LINEAR with clamp to
edge) against a numpy restatement, and the processor's interaction mode."""
import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def rescale_ref(src, W, H):
    """GL_LINEAR magnification/minification at destination pixel centres."""
    h, w = src.shape[:2]
    f32 = np.float32
    out = np.zeros((H, W, 4), np.float64)
    for y in range(H):
        vv = f32(f32(f32(y + 0.5) / f32(H)) * f32(h)) - f32(0.5)
        fv = np.floor(vv)
        av = vv - fv
        y0, y1 = int(min(max(fv, 0), h - 1)), int(min(max(fv + 1, 0), h - 1))
        for x in range(W):
            u = f32(f32(f32(x + 0.5) / f32(W)) * f32(w)) - f32(0.5)
            fu = np.floor(u)
            au = u - fu
            x0, x1 = int(min(max(fu, 0), w - 1)), int(min(max(fu + 1, 0), w - 1))
            top = src[y0, x0] + au * (src[y0, x1] - src[y0, x0])
            bot = src[y1, x0] + au * (src[y1, x1] - src[y1, x0])
            out[y, x] = top + av * (bot - top)
    return out


@pytest.mark.parametrize("w,h,W,H", [(21, 13, 64, 40), (64, 40, 21, 13), (1, 1, 5, 3), (30, 20, 90, 60)])
def test_rescale_matches_gl_linear(ctx, w, h, W, H):
    rng = np.random.default_rng(w * 100 + H)
    src = rng.uniform(0, 1, (h, w, 4)).astype(np.float32)
    ref = rescale_ref(src.astype(np.float64), W, H)
    d_src = torch.from_numpy(src).cuda()
    d_dst = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    v.image_rescale(ctx, d_src, d_dst, v.OUT_RGBA32F)
    ctx.synchronize()
    assert np.abs(d_dst.cpu().numpy() - ref).max() < 2e-6
    src8 = (src * 255).astype(np.uint8)
    d8 = torch.from_numpy(src8).cuda()
    o8 = torch.empty((H, W, 4), dtype=torch.uint8, device="cuda")
    v.image_rescale(ctx, d8, o8, v.OUT_RGBA8)
    ctx.synchronize()
    ref8 = np.floor(np.clip(rescale_ref(src8.astype(np.float64) / 255, W, H), 0, 1) * 255 + 0.5)
    assert np.abs(o8.cpu().numpy().astype(np.int32) - ref8).max() <= 1


def test_processor_interaction_coarseness(ctx):
    """Interaction mode renders at size / coarseness with rate x quality and
    rescales; the result equals that render rescaled, and the full frame is
    untouched by it."""
    from voreen_gb300.raycaster import CudaRaycaster, VolumeData
    w = synth.config2(size=(64, 60, 56), image=(96, 72))
    r = CudaRaycaster()
    r.volumeInport.setData(VolumeData(w.voxels, w.spacing))
    r.transferFunction.keys = w.tf_keys
    p = w.params(shading=v.SHADE_NONE)
    r.camera = p.camera
    r.outport.setData(np.zeros((72, 96, 4), np.float32))
    r.interactionCoarseness = 4
    r.interactionQuality = 0.5
    r.process(analytic_entry_exit=True, interacting=True)
    assert r.lastError == ""
    img = r.outport.getData()
    assert img.shape == (72, 96, 4)
    # the same coarse render by hand
    lo, hi = r.transferFunction.domain
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, 4096), (lo, hi))
    q = w.params(shading=v.SHADE_NONE, entry_exit_mode=v.EE_ANALYTIC)
    q.width, q.height, q.sampling_rate = 24, 18, p.sampling_rate * 0.5
    small, _ = v.render(ctx, vol, tf, q, None, None, v.OUT_RGBA32F)
    ref = rescale_ref(small.astype(np.float64), 96, 72)
    assert np.abs(img - ref).max() < 2e-6
    assert (img[..., 3] > 0).mean() > 0.05
    r.deinitialize()


def test_l2_read_probe(ctx):
    """The L2 peak the bench divides by: a plausible on-chip bandwidth, above
    any HBM figure, and errors as statuses."""
    g = v.measure_l2_read(ctx, 32 << 20, 10)
    assert 8000.0 < g < 200000.0
    with pytest.raises(v.VrcError):
        v.measure_l2_read(ctx, 1024, 1)
