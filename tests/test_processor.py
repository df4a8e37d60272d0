"""The processor-shaped interface (voreen_gb300.raycaster.CudaRaycaster):
port and property names and defaults as in the reference (CPU), and one
render through it against the oracle (GPU)."""
import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import synth
from voreen_gb300.raycaster import CudaRaycaster, VolumeData


def test_ports_and_property_defaults(vrc_lib):
    r = CudaRaycaster()
    assert r.volumeInport.name == "volumehandle.volumehandle"
    assert r.entryPort.name == "image.entrypoints" and r.exitPort.name == "image.exitpoints"
    assert r.outport.name == "image.output"
    assert r.samplingRate == 2.0 and r.isoValue == 0.5
    assert r.compositing == "dvr" and r.gradient == "central-differences"
    # FloatVec4Property: float32 values
    assert np.allclose(r.lightPosition, (2.3, 1.5, 1.5, 1.0), rtol=0, atol=1e-6) and r.materialShininess == 60.0
    assert r.lightAmbient[:3] == (np.float32(0.4),) * 3 and r.lightAttenuation == (1.0, 0.0, 0.0)
    assert r.className == "CudaRaycaster" and r.category == "Raycasting"
    assert not r.isReady()


def test_process_not_ready_logs_and_returns(vrc_lib):
    r = CudaRaycaster()
    r.process()
    assert "not ready" in r.lastError and not r.outport.hasData()


@pytest.mark.gpu
def test_process_renders_like_the_oracle(ctx):
    import oracle
    from helpers import oracle_entry_exit, oracle_params
    w = synth.config2(size=(64, 60, 56), image=(96, 72))
    r = CudaRaycaster()
    r.volumeInport.setData(VolumeData(w.voxels, w.spacing))
    r.transferFunction.keys = w.tf_keys
    p = w.params(shading=v.SHADE_NONE)
    r.camera = p.camera
    desc = v.make_desc(v.U16, w.dims, w.spacing)
    e, x = oracle_entry_exit(desc, p)
    r.entryPort.setData(e)
    r.exitPort.setData(x)
    r.process()
    assert r.lastError == ""
    img = r.outport.getData()
    # domain fitted to the volume's real-world min/max, width 4096 for u16
    assert r.transferFunction.width == 4096
    lo, hi = r.transferFunction.domain
    assert np.isclose(lo, w.voxels.min() / 65535.0) and np.isclose(hi, w.voxels.max() / 65535.0)
    tf = v.TransferFunction.bake(w.tf_keys, 4096)
    ref, _, _ = oracle.render(oracle.make_volume(w.voxels, w.spacing), tf, (lo, hi), oracle_params(p), e, x, 32)
    np.testing.assert_array_equal(img.view(np.uint32), ref.view(np.uint32))
    r.deinitialize()


def test_preintegrated_gpu_falls_back_with_an_error(vrc_lib):
    """cpuraycaster.cpp:123-129: pre-integrated-gpu logs an error, selects
    pre-integrated-cpu and renders nothing this call."""
    r = CudaRaycaster()
    w = synth.config1(size=(8, 8, 8), image=(4, 4))
    r.volumeInport.setData(VolumeData(w.voxels))
    r.entryPort.setData(np.zeros((4, 4, 4), np.float32))
    r.exitPort.setData(np.zeros((4, 4, 4), np.float32))
    r.classification = "pre-integrated-gpu"
    r.process()
    assert "Falling back to CPU" in r.lastError and r.classification == "pre-integrated-cpu"
    assert not r.outport.hasData()
    assert r.preIntegrationTableSize == 0 and r.gammaValue == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("classification", ["pre-integrated-cpu", "pre-integrated-approximation"])
def test_process_preintegrated_like_the_oracle(ctx, classification):
    import oracle
    from helpers import oracle_entry_exit, oracle_params
    w = synth.config1(size=(48, 40, 44), image=(80, 64))
    r = CudaRaycaster()
    r.volumeInport.setData(VolumeData(w.voxels, w.spacing))
    r.transferFunction.keys = w.tf_keys
    r.classification = classification
    p = w.params()
    r.camera = p.camera
    desc = v.make_desc(v.U8, w.dims, w.spacing)
    e, x = oracle_entry_exit(desc, p)
    r.entryPort.setData(e)
    r.exitPort.setData(x)
    r.process()
    assert r.lastError == ""
    img = r.outport.getData()
    lo, hi = r.transferFunction.domain
    step = float(np.float32(1) / (np.float32(48) * np.float32(2)))
    src = oracle.preint_source(w.tf_keys, 256)
    table = oracle.preint_table(src, step, classification.endswith("approximation"))
    tf = v.TransferFunction.bake(w.tf_keys, 256)
    ref, _, _ = oracle.render(oracle.make_volume(w.voxels, w.spacing), tf, (lo, hi),
                              oracle_params(p, preint_table=table), e, x, 32)
    np.testing.assert_array_equal(img.view(np.uint32), ref.view(np.uint32))
    r.deinitialize()


def test_brick_streaming_property_defaults(vrc_lib):
    r = CudaRaycaster()
    assert r.brickPoolPlacement == "device" and r.brickBufferSizeMB == 0
    assert r.brickUploadBudgetMB == 32 and r.useIterativeRefinement and not r.useLevelOfDetail
    r.brickPoolPlacement = "disk"
    r.volumeInport.setData(VolumeData(np.zeros((4, 4, 4), np.uint8)))
    r.process(analytic_entry_exit=True)
    assert "brick settings" in r.lastError and not r.outport.hasData()


@pytest.mark.gpu
def test_process_host_placement_refines_to_the_device_image(ctx):
    """brickPoolPlacement host with a small per-frame upload budget and the
    level of detail: process() keeps setting `invalidated` while bricks
    stream in, and the frame after the last one is the device-resident image."""
    w = synth.config2(size=(96, 80, 64), image=(160, 120))
    vd = VolumeData(w.voxels, w.spacing)

    def proc(**kw):
        r = CudaRaycaster()
        r.volumeInport.setData(vd)
        r.transferFunction.keys = w.tf_keys
        r.transferFunction.width = w.tf_width
        r.transferFunction.domain = w.domain
        r.camera = w.params().camera
        r.shading = "phong"
        r.outport.setData(np.zeros((w.height, w.width, 4), np.float32))
        for k, val in kw.items():
            setattr(r, k, val)
        return r

    dev = proc()
    dev.process(analytic_entry_exit=True)
    ref = dev.outport.getData().copy()
    host = proc(brickPoolPlacement="host", brickUploadBudgetMB=1, useLevelOfDetail=True)
    frames = 0
    host.process(analytic_entry_exit=True)
    while host.invalidated and frames < 100:
        host.process(analytic_entry_exit=True)
        frames += 1
    assert host.lastError == ""
    assert frames >= 1  # 18 bricks of 85,760 B at 12 per frame
    host.process(analytic_entry_exit=True)
    np.testing.assert_array_equal(host.outport.getData(), ref)
    dev.deinitialize()
    host.deinitialize()


def test_properties_by_id_through_the_c_shim(vrc_lib):
    """The C shim addresses properties by id like Processor::getProperty(id):
    unknown ids and wrong kinds are errors, values round-trip."""
    import ctypes as C
    r = CudaRaycaster()
    h = r._h
    assert vrc_lib.vrcp_class_name() == b"CudaRaycaster" and vrc_lib.vrcp_category() == b"Raycasting"
    f = C.c_float()
    assert vrc_lib.vrcp_set_float(h, b"samplingRate", C.c_float(4.5)) == 0
    assert vrc_lib.vrcp_get_float(h, b"samplingRate", C.byref(f)) == 0 and f.value == 4.5
    assert vrc_lib.vrcp_set_float(h, b"noSuchProperty", C.c_float(1)) != 0
    assert vrc_lib.vrcp_set_int(h, b"samplingRate", 3) != 0  # a float property
    assert vrc_lib.vrcp_set_string(h, b"compositing", b"mida") == 0 and r.compositing == "mida"
    buf = C.create_string_buffer(4)
    assert vrc_lib.vrcp_get_string(h, b"classification", buf, 4) == 0 and buf.value == b"tra"
    assert vrc_lib.vrcp_set_floatv(h, b"lightPosition", (C.c_float * 3)(1, 2, 3), 3) != 0  # vec4
    r.clipRegion = ((1, 2, 3), (10, 20, 30))
    r._push()
    v = (C.c_int * 6)()
    assert vrc_lib.vrcp_get_intv(h, b"clipRegion", v, 6) == 0 and list(v) == [1, 2, 3, 10, 20, 30]
    r.samplingRate = 25.0  # accepted, rejected by process() like Voreen's range check there
    r.volumeInport.setData(VolumeData(np.zeros((4, 4, 4), np.uint8)))
    r.process(analytic_entry_exit=True)
    assert "samplingRate" in r.lastError and not r.outport.hasData()
    r.close()


@pytest.mark.gpu
def test_preintegrated_interaction_frame(ctx):
    """Interaction mode with interactionQuality 0.5 marches at half the rate,
    so the pre-integration table is built for that step: the coarse frame
    equals a direct render with a table built for it, rescaled."""
    import oracle
    w = synth.config1(size=(48, 40, 44), image=(80, 64))
    r = CudaRaycaster()
    r.volumeInport.setData(VolumeData(w.voxels, w.spacing))
    r.transferFunction.keys = w.tf_keys
    r.classification = "pre-integrated-cpu"
    r.camera = w.params().camera
    r.outport.setData(np.zeros((64, 80, 4), np.float32))
    r.interactionCoarseness = 2
    r.interactionQuality = 0.5
    r.process(analytic_entry_exit=True, interacting=True)
    assert r.lastError == ""
    img = r.outport.getData()
    lo, hi = r.transferFunction.domain
    vol = v.Volume(ctx, w.voxels, w.spacing)
    step = v.sampling_step(vol, 1.0)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, 256), (lo, hi))
    table = v.PreIntegrationTable(ctx, oracle.preint_source(w.tf_keys, 256), step)
    tf.set_preintegration(table)
    q = w.params(entry_exit_mode=v.EE_ANALYTIC)
    q.width, q.height, q.sampling_rate, q.classification = 40, 32, 1.0, v.CLASSIFY_PREINTEGRATED
    torch = pytest.importorskip("torch")
    small = torch.empty((32, 40, 4), dtype=torch.float32, device="cuda:0")
    full = torch.empty((64, 80, 4), dtype=torch.float32, device="cuda:0")
    v.render(ctx, vol, tf, q, None, None, v.OUT_RGBA32F, small)
    v.image_rescale(ctx, small, full, v.OUT_RGBA32F)
    ctx.synchronize()
    np.testing.assert_array_equal(img, full.cpu().numpy())
    assert (img[..., 3] > 0).mean() > 0.05
    r.deinitialize()


@pytest.mark.parametrize("prop,value,msg", [
    ("compositing", "xray", "unsupported compositing"),
    ("shading", "toon", "unsupported compositing/shading"),
    ("classification", "pre-integrated-magic", "unsupported classification"),
    ("preIntegrationTableSize", 300, "unsupported classification"),
    ("interactionCoarseness", 9, "interaction settings"),
    ("interactionQuality", 0.0, "interaction settings"),
    ("brickUploadBudgetMB", 0, "brick settings"),
    ("brickBufferSizeMB", -1, "brick settings"),
])
def test_process_rejects_bad_settings_without_output(vrc_lib, prop, value, msg):
    """CPURaycaster::process logs and returns without output on a bad
    setting (cpuraycaster.cpp:125-146); no device is touched before that."""
    r = CudaRaycaster()
    r.volumeInport.setData(VolumeData(np.zeros((4, 4, 4), np.uint16)))
    setattr(r, prop, value)
    r.process(analytic_entry_exit=True)
    assert msg in r.lastError and not r.outport.hasData()
    r.close()


def test_autotuner_cache_round_trip_on_host(tmp_path):
    """The tuner's JSON cache (no GPU needed): class keys group requests by
    dtype, volume size and image size, and a loaded cache answers without
    timing."""
    import numpy as np
    from voreen_gb300 import autotune
    assert autotune.class_key(1, (512, 512, 512), 1920, 1080) == autotune.class_key(1, (500, 480, 512), 1900, 1000)
    assert autotune.class_key(1, (512, 512, 512), 1920, 1080) != autotune.class_key(0, (512, 512, 512), 1920, 1080)
    path = str(tmp_path / "t.json")
    t = autotune.Autotuner(None, cache_path=path)
    vox = np.zeros((64, 64, 64), np.uint16)
    key = autotune.class_key(1, (64, 64, 64), 256, 256)
    t.table[key] = {"tile_width": 16, "brick": 16, "skip_cell": 8, "kernel_ms": 0.5}
    t.save()
    u = autotune.Autotuner(None, cache_path=path)

    class P:
        width, height = 256, 256
    assert u.tune(vox, (1, 1, 1), None, (0, 1), P()) == t.table[key]
