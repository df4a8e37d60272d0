"""Oracle self-checks on the CPU: FP32 (faithful) against FP64, background
and degenerate-ray rules, and the synthetic workload generators."""
import numpy as np
import pytest

import oracle
import voreen_gb300 as v
from voreen_gb300 import synth

from helpers import assert_fp64_parity, oracle_entry_exit, oracle_params


def _run(w, **over):
    p = w.params(**over)
    desc = v.make_desc(v.U8 if w.voxels.dtype == np.uint8 else v.U16, w.dims, w.spacing)
    e, x = oracle_entry_exit(desc, p)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    ov = oracle.make_volume(w.voxels, w.spacing)
    op = oracle_params(p)
    o32 = oracle.render(ov, tf, w.domain, op, e, x, 32)
    o64 = oracle.render(ov, tf, w.domain, op, e, x, 64)
    return o32, o64, e


def test_fp32_vs_fp64_config1():
    w = synth.config1(image=(256, 256))
    (o32, s32, f32), (o64, s64, f64), e = _run(w)
    assert s32.sum() > 100000
    assert_fp64_parity(o32, o32, s32, f32, o64, s64, f64, v.DVR, 1.0 / (max(w.dims) * w.sampling_rate))


def test_fp32_vs_fp64_shaded_shells():
    w = synth.config2(size=(80, 80, 80), image=(160, 120))
    (o32, s32, f32), (o64, s64, f64), e = _run(w)
    assert_fp64_parity(o32, o32, s32, f32, o64, s64, f64, v.DVR, 1.0 / (max(w.dims) * w.sampling_rate))
    assert (o32[..., 3] > 0.05).mean() > 0.05


def test_background_rays_take_no_samples():
    w = synth.config1(image=(64, 64))
    (o32, s32, _), _, e = _run(w)
    bg = (e == 0).all(axis=-1)
    assert bg.any() and (s32[bg] == 0).all() and (o32[bg] == 0).all()


def test_synth_is_deterministic_and_in_range():
    a = v.synth_volume(1, v.U16, (40, 30, 20), 11)
    b = v.synth_volume(1, v.U16, (40, 30, 20), 11)
    c = v.synth_volume(1, v.U16, (40, 30, 20), 12)
    assert (a == b).all() and not (a == c).all()
    assert a.max() <= 4095
    f = v.synth_volume(0, v.F32, (16, 16, 16), 3)
    assert f.min() >= 0 and f.max() <= 1


def test_half_sample_mean_known_answers():
    """HalfSampleMean: truncating integer mean of each 2x2x2 block, indices
    clamped at odd edges; float mean in float32."""
    v = np.arange(3 * 5 * 4, dtype=np.uint16).reshape(3, 5, 4)
    h = oracle.half_sample_mean(v)
    assert h.shape == (2, 3, 2) and h.dtype == np.uint16
    assert h[0, 0, 0] == (0 + 1 + 4 + 5 + 20 + 21 + 24 + 25) // 8
    # last z block of an odd axis repeats the edge slice: z indices (2, 2)
    blk = [int(v[2, y, x]) for y in (2, 3) for x in (0, 1)] * 2
    assert h[1, 1, 0] == sum(blk) // 8
    c = np.full((7, 6, 5), 201, np.uint8)
    assert np.all(oracle.half_sample_mean(c) == 201)
    f = np.random.default_rng(3).random((4, 4, 4), dtype=np.float32)
    hf = oracle.half_sample_mean(f)
    np.testing.assert_allclose(hf[1, 0, 1], f[2:4, 0:2, 2:4].mean(), rtol=1e-6)



@pytest.mark.parametrize("comp,gamma", [(v.MIP, 0.0), (v.ISO, 0.0), (v.MOP, 0.0), (v.MIDA, -0.5), (v.MIDA, 0.5),
                                        (v.FHP, 0.0)])
def test_fp32_vs_fp64_compositing_modes(comp, gamma):
    """The oracle's FP32 path against its FP64 path for every compositing
    mode: within 1/255 on rays where both take the same discrete decisions,
    and such decisions differ on a tiny fraction of rays only."""
    w = synth.config2(size=(64, 56, 48), image=(96, 72), compositing=comp)
    (o32, s32, f32), (o64, s64, f64), e = _run(w, compositing=comp, shading=v.SHADE_NONE, mida_gamma=gamma,
                                              iso_value=0.3)
    assert s32.sum() > 10000
    assert_fp64_parity(o32, o32, s32, f32, o64, s64, f64, comp, 1.0 / (max(w.dims) * w.sampling_rate))


def test_decision_signature_explains_fp32_fp64_gaps():
    """The oracle's per-ray decision signature: on the reference's
    CPURaycaster workspace (nucleon, its 12-key TF and camera) FP32 and FP64
    differ by more than 1/255 only on rays whose decisions differ -- here a
    TF entry picked on the other side of an index rounding tie."""
    import json
    import os
    from oracle import camera as ocam
    from oracle import parity
    fix = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fixtures")
    case = json.load(open(os.path.join(fix, "cpuraycaster_vws.json")))
    vox = np.fromfile(os.path.join(fix, "nucleon.raw"), np.uint8).reshape(41, 41, 41)
    sp, off = (0.04878049,) * 3, (-0.99999994,) * 3
    cam = case["camera"]
    W, H = case["canvas"]
    inv = ocam.inverse_mvp(cam["position"], cam["focus"], cam["up"], cam["fovy"], cam["near"], cam["far"], W, H,
                           (41, 41, 41), sp, off)
    e, x = oracle.entry_exit(inv, W, H, True)
    t = [c for c in case["raycasters"] if c["classification"] == "transfer-function"][0]["tf"]
    tf = oracle.bake_tf([(k[0], tuple(k[1]), tuple(k[2])) for k in t["keys"]], t["width"])
    ov = oracle.make_volume(vox, sp, off, (255.0, 0.0))
    op = oracle.make_params(sampling_rate=2.0)
    g32, g64 = np.zeros((H, W), np.uint32), np.zeros((H, W), np.uint32)
    o32, s32, f32 = oracle.render(ov, tf, tuple(t["domain"]), op, e, x, 32, signature=g32)
    o64, s64, f64 = oracle.render(ov, tf, tuple(t["domain"]), op, e, x, 64, signature=g64)
    step = 1.0 / (41 * 2.0)
    d = np.abs(o32.astype(np.float64) - o64).max(axis=-1)
    div = parity.decision_divergent(o32, s32, f32, o64, s64, f64, v.DVR, step, sig32=g32, sig64=g64)
    assert (d > 1.0 / 255.0).any()               # this view has such rays
    assert not (d[~div] > 1.0 / 255.0).any()      # and every one of them diverges in its decisions
    assert div.sum() < 0.002 * (s32 > 0).sum()    # a handful of the hit rays
    assert (g32[s32 > 0] != 0x811C9DC5).any()     # the signatures record the entries taken
