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
