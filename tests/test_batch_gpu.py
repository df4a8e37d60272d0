"""Batched persistent render: every request of one captured launch equals
the single-request render of the same volume / TF / camera bit for bit, on
repeated replays, with per-request latencies reported."""
import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth

pytestmark = pytest.mark.gpu


def _setup(ctx, torch, n=12, seed=5):
    dims_set = ((40, 36, 33), (64, 64, 64), (96, 80, 72))
    images = ((64, 48), (96, 96), (160, 90))
    vols_raw, reqs = synth.config3(seed=seed, n=n, dims_set=dims_set, images=images)
    vols = {k: v.Volume(ctx, vox, sp) for k, (vox, sp) in vols_raw.items()}
    items, singles = [], []
    for r in reqs:
        vol = vols[r["volume"]]
        lo, hi = vol.minmax()
        tf = v.TransferFunction(ctx, v.TransferFunction.bake(r["tf_keys"], r["tf_width"]), (lo, hi))
        p = v.default_params(r["width"], r["height"])
        pos, focus, near, far = r["camera"]
        p.camera = v.make_camera(pos, focus, near=near, far=far)
        p.light_position[:] = list(r["light"])
        p.shading = v.SHADE_PHONG
        p.entry_exit_mode = v.EE_ANALYTIC
        out = torch.zeros((r["height"], r["width"], 4), dtype=torch.float32, device="cuda")
        items.append((vol, tf, p, out, v.OUT_RGBA32F))
        singles.append(v.render(ctx, vol, tf, p, None, None, v.OUT_RGBA32F)[0])
    return vols, items, singles


def test_batch_matches_single_renders(ctx):
    torch = pytest.importorskip("torch")
    vols, items, singles = _setup(ctx, torch)
    b = v.Batch(ctx, items)
    for rep in range(2):
        for it in items:
            it[3].fill_(7.0)
        b.launch()
        st, lat = b.stats()
        for (vol, tf, p, out, fmt), ref in zip(items, singles):
            got = out.cpu().numpy()
            np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
        assert st.samples > 0 and (lat > 0).all()
        assert st.latency_p50_ms <= st.latency_p99_ms <= st.latency_max_ms + 1e-6
    b.close()


def test_batch_rejects_mixed_modes(ctx):
    torch = pytest.importorskip("torch")
    vols, items, _ = _setup(ctx, torch, n=3, seed=9)
    items[1][2].compositing = v.MIP
    with pytest.raises(v.VrcError) as ei:
        v.Batch(ctx, items)
    assert ei.value.status == 4


def _request(ctx, torch, dtype, kind, dims, image, seed, shading):
    import random
    vox = v.synth_volume(kind, dtype, dims, seed)
    vol = v.Volume(ctx, vox, (1.0, 1.0, 1.0))
    lo, hi = vol.minmax()
    rng = random.Random(seed)
    keys = synth.random_trapezoid_keys(rng)
    width = v.TransferFunction.table_width(dtype)
    rgba = v.TransferFunction.bake(keys, width)
    tf = v.TransferFunction(ctx, rgba, (lo, hi))
    p = v.default_params(*image)
    pos, focus, near, far = synth.orbit_camera(dims, (1.0, 1.0, 1.0), rng.uniform(0, 360), rng.uniform(-40, 40), 1.3)
    p.camera = v.make_camera(pos, focus, near=near, far=far)
    p.light_position[:] = [*pos, 1.0]
    p.shading = shading
    p.entry_exit_mode = v.EE_ANALYTIC
    out = torch.full((image[1], image[0], 4), 7.0, dtype=torch.float32, device="cuda")
    return vox, vol, rgba, tf, p, out, (lo, hi)


@pytest.mark.parametrize("shading", [v.SHADE_NONE, v.SHADE_PHONG])
def test_batch_requests_match_oracle(ctx, shading):
    """One request per dtype (u8, u16, f32) in one launch, each against the
    FP32 oracle on the same entry/exit points (the library's analytic ones):
    unshaded bit-equal, Phong within 1e-4; and within 1/255 of FP64."""
    torch = pytest.importorskip("torch")
    import oracle
    from helpers import assert_fp64_parity, oracle_params
    reqs = [_request(ctx, torch, v.U8, synth.BLOBS, (48, 40, 36), (96, 72), 11, shading),
            _request(ctx, torch, v.U16, synth.SHELLS, (56, 48, 40), (80, 80), 12, shading),
            _request(ctx, torch, v.F32, synth.BLOBS, (40, 44, 38), (72, 96), 13, shading)]
    b = v.Batch(ctx, [(r[1], r[3], r[4], r[5], v.OUT_RGBA32F) for r in reqs])
    b.launch()
    b.stats()
    for vox, vol, rgba, tf, p, out, dom in reqs:
        got = out.cpu().numpy()
        p_buf = v.RenderParams.from_buffer_copy(p)
        p_buf.entry_exit_mode = v.EE_BUFFERS
        e, x = v.entry_exit(ctx, vol, p_buf)
        ov = oracle.make_volume(vox)
        g32 = np.zeros(e.shape[:2], np.uint32)
        g64 = np.zeros(e.shape[:2], np.uint32)
        o32, s32, fh32 = oracle.render(ov, rgba, dom, oracle_params(p), e, x, 32, signature=g32)
        assert (got[..., 3] > 0).mean() > 0.01
        if shading == v.SHADE_NONE:
            np.testing.assert_array_equal(got.view(np.uint32), o32.view(np.uint32))
        else:
            assert np.abs(got - o32).max() <= 1e-4
        o64, s64, fh64 = oracle.render(ov, rgba, dom, oracle_params(p), e, x, 64, signature=g64)
        assert_fp64_parity(got, o32, s32, fh32, o64, s64, fh64, v.DVR, 1.0 / (max(vox.shape) * p.sampling_rate),
                           shaded=shading != v.SHADE_NONE, sigs=(g32, g64))
    b.close()


def test_batch_isolates_poisoned_requests(ctx):
    """A request that fails its checks returns its own status and is left out;
    the other requests of the launch complete bit-equal to their single
    renders, and the poisoned outputs are not written."""
    torch = pytest.importorskip("torch")
    vols, items, singles = _setup(ctx, torch, n=8, seed=21)
    items = [list(it) for it in items]
    items[1][1] = None                        # no transfer function
    items[3][2] = v.RenderParams.from_buffer_copy(items[3][2])
    items[3][2].width = 0                     # invalid image size
    items[5][2] = v.RenderParams.from_buffer_copy(items[5][2])
    items[5][2].compositing = v.MIP           # another compositing mode than the batch's
    items[6][2] = v.RenderParams.from_buffer_copy(items[6][2])
    items[6][2].entry_exit_mode = v.EE_BUFFERS  # batches march analytic entry/exit only
    items = [tuple(it) for it in items]
    with pytest.raises(v.VrcError):
        v.Batch(ctx, items)                   # all-or-nothing form
    b = v.Batch(ctx, items, isolate=True)
    expect = {1: 1, 3: 1, 5: 4, 6: 4}
    assert b.status == [expect.get(i, 0) for i in range(len(items))]
    for it in items:
        it[3].fill_(7.0)
    b.launch()
    st, lat = b.stats()
    for i, ((vol, tf, p, out, fmt), ref) in enumerate(zip(items, singles)):
        got = out.cpu().numpy()
        if i in expect:
            assert (got == 7.0).all() and lat[i] == -1.0
        else:
            np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
            assert lat[i] > 0
    b.close()


def test_autotuner_picks_fastest_timed_candidate(ctx, tmp_path):
    """The tuned settings are the fastest of the candidates it timed, they do
    not change the image, and the JSON cache round-trips (a second tuner
    answers from the cache without timing anything)."""
    torch = pytest.importorskip("torch")
    from voreen_gb300 import autotune
    w = synth.config2(size=(96, 80, 72), image=(160, 120))
    rgba = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    p = w.params()
    path = str(tmp_path / "tune.json")
    tuner = autotune.Autotuner(ctx, cache_path=path, frames=2)
    best = tuner.tune(w.voxels, w.spacing, rgba, w.domain, p)
    key = autotune.class_key(v.U16, w.dims, w.width, w.height)
    timed = tuner.timings[key]
    assert len(timed) == sum(1 for b_ in autotune.BRICKS for c in autotune.SKIP_CELLS if c <= b_) * len(
        autotune.TILE_WIDTHS)
    fastest = min(timed, key=lambda t: t[3])
    assert (best["tile_width"], best["brick"], best["skip_cell"], best["kernel_ms"]) == fastest
    assert best["skip_cell"] <= best["brick"]
    tuner.save()
    again = autotune.Autotuner(ctx, cache_path=path)

    def no_timing(*a, **k):
        raise AssertionError("a cached class was timed again")

    again._time = no_timing
    assert again.tune(w.voxels, w.spacing, rgba, w.domain, w.params()) == best
    # the tuned launch shape renders the same image as the defaults
    q = w.params()
    q.entry_exit_mode = v.EE_ANALYTIC
    vol_d = v.Volume(ctx, w.voxels, w.spacing)
    vol_t = v.Volume(ctx, w.voxels, w.spacing, brick_size=best["brick"])
    tf = v.TransferFunction(ctx, rgba, w.domain)
    ref, _ = v.render(ctx, vol_d, tf, q, None, None, v.OUT_RGBA32F)
    q.tile_width, q.skip_cell_size = best["tile_width"], best["skip_cell"]
    got, _ = v.render(ctx, vol_t, tf, q, None, None, v.OUT_RGBA32F)
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
