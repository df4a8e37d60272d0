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
