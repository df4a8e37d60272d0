"""vrc_render_noalloc through the C ABI.

This entry point exists for callers that cannot allocate device memory while
they render (real-time loops, hosts with their own fixed device-memory
pool): it keeps its scratch in a fixed array inside the library. Its frames
must equal vrc_render's (same kernels, the same TF values: bit-equal), on
consecutive calls that share that array, also for a brick pool in host
memory, and a request beyond the array's capacity must be refused with
VRC_ERR_SCRATCH_LIMIT. Collected last so that a failure here leaves every
other test already run.
"""
import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth

pytestmark = pytest.mark.gpu


def _frame_pair(ctx, torch, w, p, out_format=v.OUT_RGBA32F):
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    e, x = v.entry_exit(ctx, vol, p)
    e_d = torch.from_numpy(e).cuda()
    x_d = torch.from_numpy(x).cuda()
    dt = torch.float32 if out_format == v.OUT_RGBA32F else torch.uint8
    ref = torch.zeros((p.height, p.width, 4), dtype=dt, device="cuda")
    got = torch.full((p.height, p.width, 4), 7, dtype=dt, device="cuda")
    torch.cuda.synchronize()
    v.render(ctx, vol, tf, p, e_d, x_d, out_format, ref)
    ctx.synchronize()
    v.render_noalloc(vol, tf, p, e_d, x_d, got, out_format, ctx.stream)
    ctx.synchronize()
    return ref.cpu().numpy(), got.cpu().numpy(), (vol, tf)


def test_noalloc_matches_render_on_consecutive_calls(ctx):
    torch = pytest.importorskip("torch")
    # call 1: shaded DVR with a 4096-entry TF and the default skip cells (4^3 with the distance field)
    w1 = synth.config2(size=(96, 88, 80), image=(200, 150))
    p1 = w1.params()
    ref1, got1, keep1 = _frame_pair(ctx, torch, w1, p1)
    assert (ref1[..., 3] > 0).any()
    np.testing.assert_array_equal(got1.view(np.uint32), ref1.view(np.uint32))
    # call 2 reuses the same scratch with a different TF width, mode and
    # skip-cell grid: nothing of call 1 may leak into it
    w2 = synth.config1(size=(64, 60, 56), image=(160, 120))
    p2 = w2.params(compositing=v.MIP, skip_cell_size=16)
    ref2, got2, keep2 = _frame_pair(ctx, torch, w2, p2, v.OUT_RGBA8)
    assert (ref2[..., 3] > 0).any()
    np.testing.assert_array_equal(got2, ref2)


def test_noalloc_refuses_requests_beyond_its_scratch(ctx):
    torch = pytest.importorskip("torch")
    # 1040^3 voxels: the default takes 8^3 cells (4^3 would be 260^3), and 130^3 cells > VRC_NOALLOC_MAX_CELLS
    vox = np.zeros((1040, 1040, 1040), np.uint8)
    vox[500:540, 500:540, 500:540] = 200
    vol = v.Volume(ctx, vox)
    del vox
    tf = v.TransferFunction(ctx, v.TransferFunction.bake([(0.0, (0, 0, 0, 0)), (1.0, (255, 255, 255, 255))], 256))
    p = v.default_params(32, 32)
    p.entry_exit_mode = v.EE_ANALYTIC
    p.camera = v.make_camera((520, 520, 3000), (520, 520, 520), near=1.0, far=5000.0)
    out = torch.zeros((32, 32, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(v.VrcError) as ei:
        v.render_noalloc(vol, tf, p, None, None, out, v.OUT_RGBA32F, ctx.stream)
    assert ei.value.status == 8
    assert v.NOALLOC_MAX_CELLS == 2097152
    # within the limit (16^3 cells: 65^3 of them) the same volume renders
    p.skip_cell_size = 16
    v.render_noalloc(vol, tf, p, None, None, out, v.OUT_RGBA32F, ctx.stream)
    ctx.synchronize()
    ref, _ = v.render(ctx, vol, tf, p, None, None, v.OUT_RGBA32F)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    vol.close()


def test_noalloc_host_placed_pool(ctx):
    """A brick pool in pinned host memory is read in place: the frame equals
    vrc_render's of the same volume (which reads it through its device brick
    cache) and of the device-resident volume."""
    torch = pytest.importorskip("torch")
    w = synth.config2(size=(80, 72, 64), image=(160, 120))
    p = w.params()
    p.entry_exit_mode = v.EE_ANALYTIC
    host = v.Volume(ctx, w.voxels, w.spacing, placement=v.PLACE_HOST, brick_size=16)
    dev = v.Volume(ctx, w.voxels, w.spacing, brick_size=16)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    ref_dev, _ = v.render(ctx, dev, tf, p, None, None, v.OUT_RGBA32F)
    ref_host, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
    for _ in range(2):
        got = torch.full((p.height, p.width, 4), 3.0, dtype=torch.float32, device="cuda")
        v.render_noalloc(host, tf, p, None, None, got, v.OUT_RGBA32F, ctx.stream)
        ctx.synchronize()
        g = got.cpu().numpy()
        assert (g[..., 3] > 0).any()
        np.testing.assert_array_equal(g.view(np.uint32), ref_host.view(np.uint32))
        np.testing.assert_array_equal(g.view(np.uint32), ref_dev.view(np.uint32))
    host.close()
    dev.close()


def test_noalloc_rejects_handles_of_two_contexts(ctx):
    torch = pytest.importorskip("torch")
    other = v.Context(0)
    try:
        w = synth.config1(size=(32, 32, 32), image=(32, 32))
        vol = v.Volume(ctx, w.voxels, w.spacing)
        tf = v.TransferFunction(other, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
        p = w.params()
        p.entry_exit_mode = v.EE_ANALYTIC
        out = torch.zeros((32, 32, 4), dtype=torch.float32, device="cuda")
        with pytest.raises(v.VrcError) as ei:
            v.render_noalloc(vol, tf, p, None, None, out, v.OUT_RGBA32F, ctx.stream)
        assert ei.value.status == 1
        tf.close()
        vol.close()
    finally:
        other.close()
