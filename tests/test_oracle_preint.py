"""CPU checks of the oracle's pre-integration table (PreIntegrationTable::
computeTable) and of the extra compositing modes on small hand-made cases.
The reference's table builder needs its GL texture stack to compile, so
these are known-answer and property checks, not reference-produced vectors."""
import numpy as np
import pytest

import oracle


def _source(res, entries):
    """res x RGBA8 with the given {index: (r, g, b, a)} entries, zero elsewhere."""
    src = np.zeros((res, 4), np.uint8)
    for i, c in entries.items():
        src[i] = c
    return src


def test_diagonal_is_the_opacity_corrected_tf(orc):
    rng = np.random.default_rng(1)
    src = rng.integers(0, 256, size=(64, 4)).astype(np.uint8)
    step = np.float32(1 / 700)
    for integral in (False, True):
        t = orc.preint_table(src, float(step), integral)
        d = t[np.arange(64), np.arange(64)]
        a = src[:, 3].astype(np.float32) / np.float32(255)
        corr = np.float32(1) - np.power(np.float32(1) - a, np.float32(step * np.float32(200)))
        np.testing.assert_allclose(d[:, 3], corr, rtol=2e-6, atol=1e-7)
        np.testing.assert_allclose(d[:, :3], src[:, :3].astype(np.float32) / 255, rtol=0, atol=1e-7)


def test_single_entry_segment(orc):
    """Only entry 40 is visible: every segment covering it has that entry's
    colour and opacity 1 - (1 - a)^(200 step / (k + 1)); segments missing it
    are empty."""
    res, a8 = 128, 180
    src = _source(res, {40: (200, 100, 50, a8)})
    step = 1 / 512
    t = orc.preint_table(src, step, False)
    for sb, sf in [(10, 70), (70, 10), (40, 41), (39, 40), (0, 127)]:
        k = abs(sb - sf)
        a = 1 - (1 - a8 / 255) ** (200 * step / (k + 1))
        assert t[sb, sf, 3] == pytest.approx(a, rel=1e-5)
        np.testing.assert_allclose(t[sb, sf, :3], np.array([200, 100, 50]) / 255, atol=2e-6)
    for sb, sf in [(0, 39), (41, 127), (50, 60)]:
        assert np.all(t[sb, sf] == 0)


def test_constant_tf_segment_matches_one_sample(orc):
    """A constant TF composited over k + 1 entries with the 1/(k + 1) correction
    gives the one-sample opacity 1 - (1 - a)^(200 step) (no early termination
    below 0.95), and the colour of the TF."""
    res = 64
    src = np.tile(np.array([[30, 160, 220, 12]], np.uint8), (res, 1))
    step = 1 / 256
    t = orc.preint_table(src, step, False)
    a1 = 1 - (1 - 12 / 255) ** (200 * step)
    for sb, sf in [(3, 9), (60, 1), (0, 63)]:
        assert t[sb, sf, 3] == pytest.approx(a1, rel=2e-4)  # FP32 sums of k + 1 small terms
        np.testing.assert_allclose(t[sb, sf, :3], np.array([30, 160, 220]) / 255, atol=2e-6)


def test_integral_table_constant_tf_closed_form(orc):
    """Integral functions of a constant TF: alpha = 1 - exp(-a * 200 step),
    colour = c * a * 200 step / alpha."""
    res = 64
    src = np.tile(np.array([[30, 160, 220, 40]], np.uint8), (res, 1))
    step = 1 / 300
    t = orc.preint_table(src, step, True)
    a = 40 / 255
    alpha = 1 - np.exp(-a * 200 * step)
    col = np.array([30, 160, 220]) / 255 * a * 200 * step / alpha
    for sb, sf in [(3, 9), (60, 1), (0, 63)]:
        assert t[sb, sf, 3] == pytest.approx(alpha, rel=1e-4)
        np.testing.assert_allclose(t[sb, sf, :3], np.clip(col, 0, 1), rtol=1e-4)


def test_early_termination_in_the_table(orc):
    """Compositing stops once the segment's opacity reaches 0.95."""
    res = 32
    src = np.tile(np.array([[255, 0, 0, 255]], np.uint8), (res, 1))
    src[20:, :3] = (0, 255, 0)
    t = orc.preint_table(src, 1.0, False)  # step 1: every entry nearly opaque
    assert t[31, 0, 3] >= 0.95
    assert t[31, 0, 1] == 0.0  # stopped before the green entries


def test_preint_source_thresholds(orc):
    keys = [(0.0, (10, 20, 30, 40)), (1.0, (250, 240, 230, 220))]
    res = 100
    full = orc.preint_source(keys, res)
    cut = orc.preint_source(keys, res, threshold=(0.2, 0.7))
    assert np.all(cut[:20] == 0) and np.all(cut[70:] == 0)
    np.testing.assert_array_equal(cut[20:70], full[20:70])
    # the texture bake keeps entry iround(0.7 * res) = 70; the table source does not
    tex = orc.bake_tf(keys, res, threshold=(0.2, 0.7))
    np.testing.assert_array_equal(tex[70], full[70])


def _tiny_case(orc, compositing, keys=None, **kw):
    rng = np.random.default_rng(5)
    vox = rng.integers(0, 256, size=(6, 7, 8), dtype=np.uint8)
    ov = orc.make_volume(vox)
    keys = keys or [(0.0, (0, 0, 255, 0)), (0.3, (0, 255, 0, 60)), (1.0, (255, 0, 0, 200))]
    tf = orc.bake_tf(keys, 256)
    e = np.zeros((1, 2, 4), np.float32)
    x = np.zeros((1, 2, 4), np.float32)
    e[0, 0] = (0.05, 0.5, 0.5, 1)
    x[0, 0] = (0.95, 0.45, 0.55, 1)
    e[0, 1] = (0.5, 0.02, 0.3, 1)
    x[0, 1] = (0.5, 0.98, 0.7, 1)
    p = orc.make_params(compositing=compositing, **kw)
    return orc.render(ov, tf, (0.0, 1.0), p, e, x, 64)


def test_fhp_returns_the_first_visible_position(orc):
    out, s, fh = _tiny_case(orc, orc.FHP)
    assert np.all(out[..., 3] == 1)
    # the first-hit position lies on the ray segment
    t = fh[0, 0]
    p0, p1 = np.array([0.05, 0.5, 0.5]), np.array([0.95, 0.45, 0.55])
    d = (p1 - p0) / np.linalg.norm(p1 - p0)
    np.testing.assert_allclose(out[0, 0, :3], p0 + t * d, atol=1e-12)


def test_fhn_is_a_unit_normal_mapped_to_unit_range(orc):
    """Visible only above 0.6, so the first hit is past the entry point (at
    t = 0 the normal comes from neighbouring entry points, degenerate in a
    2 x 1 image)."""
    out, _, fh = _tiny_case(orc, orc.FHN, keys=[(0.0, (0, 0, 0, 0)), (0.6, (0, 0, 0, 0)), (1.0, (255, 0, 0, 200))])
    assert np.all(fh > 0)
    n = out[..., :3] * 2 - 1
    np.testing.assert_allclose(np.linalg.norm(n, axis=-1), 1.0, atol=1e-9)


def test_mida_gamma_limits(orc):
    """gamma = 1 is MIP of the opacity-corrected colour (the MIDA half is
    weighted 0); MOP keeps the most opaque sample."""
    mida1, s1, _ = _tiny_case(orc, orc.MIDA, mida_gamma=1.0)
    mip, s2, _ = _tiny_case(orc, orc.MIP)
    np.testing.assert_array_equal(s1, s2)  # neither terminates early
    np.testing.assert_allclose(mida1[..., :3], mip[..., :3], atol=1e-12)
    mop, _, _ = _tiny_case(orc, orc.MOP)
    assert np.all(mop[..., 3] >= mip[..., 3] - 1e-12)
