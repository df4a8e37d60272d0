"""Parity at the benchmark's full size: 512^3 u16 CT-like shells, spacing
(0.7, 0.7, 1.0), 4096-entry TF, 1920x1080, 2 samples/voxel -- the frame the
headline number is measured on -- against the CPU oracle on the same inputs
(the loop of modules/base/processors/render/cpuraycaster.cpp:239-317).

Phong DVR: within 1e-4 of the FP32 oracle with equal sample counts, and
within 1/255 of the FP64 oracle on every ray where FP32 and FP64 take the
same discrete decisions (the others are counted and reported). MIP: bit-equal
to the FP32 oracle, and the same FP64 bar."""
import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth

from helpers import Case, assert_fp64_parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2(ctx):
    w = synth.config2()
    assert w.dims == (512, 512, 512) and (w.width, w.height) == (1920, 1080)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, w.params(), w.spacing)
    yield w, c
    c.vol.close()
    c.tf.close()


def test_c2_phong_dvr_full_frame(c2):
    w, c = c2
    c.params.compositing, c.params.shading = v.DVR, v.SHADE_PHONG
    img, st = c.gpu()
    o32, s32, fh32 = c.oracle(32)
    assert st.samples == s32.sum()
    assert st.samples_shaded > 1_000_000
    assert np.abs(img - o32).max() <= 1e-4
    o64, s64, fh64 = c.oracle(64)
    assert_fp64_parity(img, o32, s32, fh32, o64, s64, fh64, v.DVR, c.step, shaded=True,
                       label="C2 512^3 u16 1920x1080 Phong DVR (full frame)", sigs=c.sigs)


def test_c2_mip_full_frame(c2):
    w, c = c2
    c.params.compositing, c.params.shading = v.MIP, v.SHADE_NONE
    img, st = c.gpu()
    o32, s32, fh32 = c.oracle(32)
    assert st.samples == s32.sum()
    np.testing.assert_array_equal(np.ascontiguousarray(img).view(np.uint32), o32.view(np.uint32))
    o64, s64, fh64 = c.oracle(64)
    assert_fp64_parity(img, o32, s32, fh32, o64, s64, fh64, v.MIP, c.step,
                       label="C2 512^3 u16 1920x1080 MIP (full frame)", sigs=c.sigs)
