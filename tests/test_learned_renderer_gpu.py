"""The learned render path end to end (LearnedRenderer): the probe's fallback
decision, the fallback frame, and what the trained network gains over the
method without it (bilinear upsampling of the same half-resolution march),
compared with the plain full-rate render on held-out volumes."""
import math
import os

import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "voreen_gb300", "weights",
                       "upsampler_ct.npz")


@pytest.fixture(scope="module")
def net(vrc_lib):
    from voreen_gb300 import learned
    n = learned.UNet(seed=0)
    n.load(WEIGHTS)
    return n


def _scene(ctx, size=192, image=(480, 272), seed=3):
    w = synth.config2(seed=seed, size=(size,) * 3, image=image)
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    return w, vol, tf


def test_forced_fallback_is_the_plain_frame(ctx, net):
    """With an unreachable PSNR bound every frame falls back, and the frame is
    bit-equal to the plain render (vrc_render) of the same parameters."""
    torch = pytest.importorskip("torch")
    from voreen_gb300 import learned
    w, vol, tf = _scene(ctx)
    r = learned.LearnedRenderer(ctx, net, psnr_bound=math.inf)
    p = w.params()
    for _ in range(2):
        frame, info = r.render(vol, tf, p)
        torch.cuda.synchronize()
        assert info["fallback"]
        ref, _ = learned.plain_frame(ctx, vol, tf, p)
        assert torch.equal(frame, ref)
    assert r.fallbacks == r.frames == 2


def test_no_fallback_gives_the_network_frame(ctx, net):
    """With no bound the network's frame is returned: it differs from the
    plain render but stays close to it."""
    torch = pytest.importorskip("torch")
    from voreen_gb300 import learned
    w, vol, tf = _scene(ctx)
    r = learned.LearnedRenderer(ctx, net, psnr_bound=-math.inf)
    p = w.params()
    frame, info = r.render(vol, tf, p)
    torch.cuda.synchronize()
    ref, _ = learned.plain_frame(ctx, vol, tf, p)
    assert not info["fallback"] and r.fallbacks == 0
    assert not torch.equal(frame, ref)
    assert learned.psnr(frame, ref) > 25.0


def test_fallback_count_follows_the_probe(ctx, net):
    """Over a sequence of views the renderer falls back exactly when the
    probe's frame estimate is below the bound, and counts it."""
    torch = pytest.importorskip("torch")
    from voreen_gb300 import learned
    w, vol, tf = _scene(ctx)
    r = learned.LearnedRenderer(ctx, net, psnr_bound=40.0)
    decisions = []
    for k in range(6):
        pos, focus, near, far = synth.orbit_camera(w.dims, w.spacing, 20.0 + 50.0 * k, 10.0 * (k % 3) - 10.0, 1.25)
        p = w.params()
        p.camera = v.make_camera(pos, focus, near=near, far=far)
        p.light_position[:] = [*pos, 1.0]
        frame, info = r.render(vol, tf, p)
        assert info["fallback"] == (info["frame_psnr_estimate"] < 40.0)
        if info["fallback"]:
            ref, _ = learned.plain_frame(ctx, vol, tf, p)
            assert torch.equal(frame, ref)
        decisions.append(info["fallback"])
    assert r.frames == 6 and r.fallbacks == sum(decisions)


def test_network_beats_bilinear_on_held_out_volumes(ctx, net):
    """The trained network against the method without it: on held-out seeds
    (volumes and views it was not trained on) its frame is closer to the
    plain full-rate render than the bilinear upsampling of the same
    half-resolution, half-rate march, by a margin."""
    from voreen_gb300 import learned
    vols = []
    for s in (100, 101):
        vox = v.synth_volume(synth.SHELLS, v.U16, (512, 512, 512), 4000 + s)
        vols.append((v.Volume(ctx, vox, (0.7, 0.7, 1.0)), vox, (0.7, 0.7, 1.0)))
    ev = learned.evaluate(ctx, net, vols, views=3, seed=777)
    gain = [e["psnr_net"] - e["psnr_bilinear"] for e in ev]
    assert min(gain) > 0.0, gain
    assert np.mean(gain) > 1.0, gain
    for vol, _, _ in vols:
        vol.close()


def test_tube_weights_beat_bilinear_on_held_out_tube_volumes(ctx):
    """The tube-family weights (trained on 1024x1024x512 volumes of 125
    tubes, seeds 6000-6003) on held-out tube volumes and views: closer to the
    plain render than bilinear upsampling of the same march, by at least
    0.5 dB on average. Thin tubes at half resolution stay well below the
    40 dB bound (about 34 dB), which is why large tube frames fall back."""
    from voreen_gb300 import learned
    net_t = learned.UNet(seed=0)
    net_t.load(os.path.join(os.path.dirname(WEIGHTS), "upsampler_tubes.npz"))
    vols = []
    for s in (100, 101):
        dims = (1024, 1024, 512)
        vox = v.synth_tubes_device(dims, 125, 6000 + s)
        vol = v.Volume(ctx, vox, (1.0, 1.0, 1.0))
        vols.append((vol, {"dims": dims, "minmax": vol.minmax()}, (1.0, 1.0, 1.0)))
        del vox
    ev = learned.evaluate(ctx, net_t, vols, views=4, seed=778, view_fn=learned.random_view_tubes)
    gain = [e["psnr_net"] - e["psnr_bilinear"] for e in ev]
    assert min(gain) > 0.0, gain
    assert np.mean(gain) > 0.5, gain
    assert max(e["psnr_net"] for e in ev) < 40.0
    for vol, _, _ in vols:
        vol.close()


def test_probe_beyond_the_noalloc_scratch_renders_on_the_context_stream(ctx, net):
    """The probe tile renders on a side stream through vrc_render_noalloc,
    whose fixed scratch holds at most NOALLOC_MAX_CELLS empty-space cells.
    A volume with more cells (here 4^3 cells of a 520^3 volume: 2,197,000)
    makes vrc_render_noalloc return VRC_ERR_SCRATCH_LIMIT; the renderer then
    renders the tile on the context stream, and the fallback frame is still
    the plain render."""
    torch = pytest.importorskip("torch")
    from voreen_gb300 import learned
    w = synth.config2(seed=5, size=(520, 520, 520), image=(320, 192))
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    p = w.params(skip_cell_size=4, entry_exit_mode=v.EE_ANALYTIC)
    assert (520 // 4) ** 3 > v.NOALLOC_MAX_CELLS
    ref = torch.zeros((w.height, w.width, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(v.VrcError, match="SCRATCH_LIMIT"):
        v.render_noalloc(vol, tf, p, None, None, ref)
    r = learned.LearnedRenderer(ctx, net, psnr_bound=math.inf)
    frame, info = r.render(vol, tf, p)
    torch.cuda.synchronize()
    assert info["fallback"]
    assert r._no_side.get(vol.handle.value)
    plain, _ = learned.plain_frame(ctx, vol, tf, p)
    assert torch.equal(frame, plain)
    tf.close()
    vol.close()
