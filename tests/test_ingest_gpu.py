"""Volume ingest on the GPU: a .vvd file streamed through pinned chunks into
the bricked layout renders exactly as the same voxels uploaded from memory."""
import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,path_list", [(v.U16, False), (v.U8, True), (v.F32, False)])
def test_load_vvd_renders_like_memory_upload(ctx, tmp_path, dtype, path_list):
    w = synth.config2(size=(70, 61, 53), image=(120, 90))
    vox = {v.U16: w.voxels, v.U8: (w.voxels >> 4).astype(np.uint8),
           v.F32: (w.voxels / 4095.0).astype(np.float32)}[dtype]
    rwm = (2.0, -0.1)
    v.write_vvd(str(tmp_path / "vol.vvd"), vox, spacing=w.spacing, offset=(0.5, -1.0, 2.0), rwm=rwm,
                path_list=path_list)
    a = v.Volume.load_vvd(ctx, str(tmp_path / "vol.vvd"))
    b = v.Volume(ctx, vox, w.spacing, (0.5, -1.0, 2.0), rwm)
    assert a.dims == b.dims and a.minmax() == b.minmax()
    scale = {v.U8: 255.0, v.U16: 65535.0, v.F32: 1.0}[dtype]
    assert a.minmax() == pytest.approx((float(np.float32(vox.min() / scale)), float(np.float32(vox.max() / scale))))
    lo, hi = a.minmax()
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, v.TransferFunction.table_width(dtype)),
                            (lo * rwm[0] + rwm[1], hi * rwm[0] + rwm[1]))
    p = w.params(entry_exit_mode=v.EE_ANALYTIC)
    ia, _ = v.render(ctx, a, tf, p, None, None, v.OUT_RGBA32F)
    ib, _ = v.render(ctx, b, tf, p, None, None, v.OUT_RGBA32F)
    np.testing.assert_array_equal(ia.view(np.uint32), ib.view(np.uint32))
    assert (ia[..., 3] > 0).mean() > 0.05


def test_load_vvd_errors(ctx, tmp_path):
    vox = np.zeros((4, 4, 4), np.uint8)
    v.write_vvd(str(tmp_path / "short.vvd"), vox)
    (tmp_path / "short.raw").write_bytes(b"\0" * 10)   # shorter than 4^3 voxels
    with pytest.raises(v.VrcError, match="INVALID_ARG"):
        v.Volume.load_vvd(ctx, str(tmp_path / "short.vvd"))
    with pytest.raises(v.VrcError, match="NOT_READY"):
        v.Volume.load_vvd(ctx, str(tmp_path / "missing.vvd"))
