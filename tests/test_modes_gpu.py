"""GPU parity of the compositing modes beyond DVR / MIP / ISO (MOP, MIDA,
first-hit position and normal, mod_compositing.frag:97-196) and of
pre-integrated classification (PreIntegrationTable, cpuraycaster.cpp:255-261):
tables equal to the oracle's bit for bit, renders equal to the FP32 oracle
bit for bit when unshaded, empty-space skipping exact in every mode."""
import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth

from helpers import Case

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _shells(ctx, comp, shading=v.SHADE_NONE, size=(96, 80, 72), image=(200, 150), **over):
    w = synth.config2(size=size, image=image)
    p = w.params(shading=shading)
    p.compositing = comp
    for k, val in over.items():
        setattr(p, k, val)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    return Case(ctx, w.voxels, tf, w.domain, p, w.spacing)


MODES = [(v.MOP, 0.0), (v.MIDA, -0.5), (v.MIDA, 0.0), (v.MIDA, 0.6), (v.FHP, 0.0), (v.FHN, 0.0)]


@pytest.mark.parametrize("comp,gamma", MODES)
def test_extra_modes_unshaded_bit_exact(ctx, comp, gamma):
    c = _shells(ctx, comp, mida_gamma=gamma)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32)
    assert st.samples == s32.sum()
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert (img[..., 3] > 0).mean() > 0.05  # the shells cover ~11 % of this frame


@pytest.mark.parametrize("comp,gamma", [(v.MOP, 0.0), (v.MIDA, 0.3)])
def test_extra_modes_phong(ctx, comp, gamma):
    c = _shells(ctx, comp, shading=v.SHADE_PHONG, mida_gamma=gamma)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32)
    assert st.samples == s32.sum()
    assert np.abs(img - o32).max() <= 1e-4


@pytest.mark.parametrize("comp,gamma", MODES)
def test_extra_modes_skipping_exact(ctx, comp, gamma):
    c = _shells(ctx, comp, size=(130, 128, 127), image=(256, 192), mida_gamma=gamma)
    a, sa = c.gpu(empty_space_skipping=1)
    b, sb = c.gpu(empty_space_skipping=0)
    np.testing.assert_array_equal(_bits(a), _bits(b))
    assert sa.samples == sb.samples and sa.samples_fetched < sb.samples_fetched


@pytest.mark.parametrize("res,integral", [(256, False), (1000, False), (1024, True), (64, True)])
def test_preint_table_equals_oracle(ctx, orc, res, integral):
    w = synth.config2(size=(64, 64, 64), image=(32, 32))
    src = v.PreIntegrationTable.bake_source(w.tf_keys, res)
    np.testing.assert_array_equal(src, orc.preint_source(w.tf_keys, res))
    step = float(np.float32(1.0) / (np.float32(512) * np.float32(2.0)))
    t = v.PreIntegrationTable(ctx, src, step, integral)
    got = t.download()
    ref = orc.preint_table(src, t.step, integral)
    np.testing.assert_array_equal(_bits(got), _bits(ref))


def _preint_case(ctx, orc, integral, vol_kind, shading=v.SHADE_NONE, res=0, rate=None):
    if vol_kind == "blobs":
        w = synth.config1(size=(64, 72, 56), image=(160, 128))
    else:
        w = synth.config2(size=(96, 80, 72), image=(200, 150))
    p = w.params(shading=shading)
    if rate is not None:
        p.sampling_rate = rate
    p.classification = v.CLASSIFY_PREINTEGRATED
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, p, w.spacing)
    n = v.PreIntegrationTable.resolution(w.tf_width, res)
    src = v.PreIntegrationTable.bake_source(w.tf_keys, n)
    table = v.PreIntegrationTable(ctx, src, v.sampling_step(c.vol, p.sampling_rate), integral)
    c.tf.set_preintegration(table)
    return c, table


@pytest.mark.parametrize("integral,vol_kind,rate", [(False, "blobs", None), (True, "blobs", None),
                                                    (False, "shells", None), (True, "shells", None),
                                                    (False, "shells", 0.8), (False, "shells", 1.0)])
def test_preint_render_bit_exact(ctx, orc, integral, vol_kind, rate):
    """Rates above 1 let empty-to-empty segments skip (a step moves less than a
    voxel per axis); at rate <= 1 the first sample of every empty run is
    classified as usual."""
    c, table = _preint_case(ctx, orc, integral, vol_kind, rate=rate)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32, preint_table=table.download())
    assert st.samples == s32.sum()
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert (img[..., 3] > 0).mean() > 0.03  # ~6 % (blobs) and more (shells) of the frame are hit
    # skipping stays exact with the previous-sample dependence
    b, sb = c.gpu(empty_space_skipping=0)
    np.testing.assert_array_equal(_bits(img), _bits(b))
    assert sb.samples == st.samples


def test_preint_render_phong(ctx, orc):
    c, table = _preint_case(ctx, orc, False, "shells", shading=v.SHADE_PHONG, res=512)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32, preint_table=table.download())
    assert st.samples == s32.sum()
    assert np.abs(img - o32).max() <= 1e-4


def test_preint_and_mode_errors(ctx, orc):
    c, table = _preint_case(ctx, orc, False, "blobs")
    p = c.params
    # a table built for another step size is refused
    wrong = v.PreIntegrationTable(ctx, table.source, table.step * 2)
    c.tf.set_preintegration(wrong)
    with pytest.raises(v.VrcError, match="INVALID_ARG"):
        c.gpu()
    c.tf.set_preintegration(None)
    with pytest.raises(v.VrcError, match="NOT_READY"):
        c.gpu()
    c.tf.set_preintegration(table)
    with pytest.raises(v.VrcError, match="INVALID_ARG"):
        c.gpu(compositing=v.MIP)  # pre-integration is DVR only
    p.compositing = v.DVR
    p.classification = 7
    with pytest.raises(v.VrcError, match="INVALID_ARG"):
        c.gpu()
    p.classification = v.CLASSIFY_TF
    with pytest.raises(v.VrcError, match="INVALID_ARG"):
        c.gpu(compositing=9)
    p.compositing = v.DVR
