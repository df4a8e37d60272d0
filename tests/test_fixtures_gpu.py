"""The reference's own fixed-input cases, rendered on the GPU against the CPU
oracle: Voreen's sample volumes nucleon (41^3 uint8), walnut
(128x96x114 uint16) and vessel-tree-noisy (101^3 uint8) loaded through
vrc_volume_load_vvd with their sample transfer functions (a key preset for
the vessel tree) read by vrc_tf_read_tfi, and the CPURaycaster regression
workspace modules/base/test/render/cpuraycaster.vws (nucleon, its 12-key TF,
camera and canvas; TF and pre-integrated classification). The files are
copies made by tests/golden/make_fixtures.py.

The oracle side states the reference's loading rules itself: a .vvd without
a RealWorldMapping gets the denormalizing mapping of its format
(modules/core/io/vvdvolumereader.cpp:102-120; uint8 -> 255, uint16 -> 65535),
and the entry/exit points of MeshEntryExitPoints are rendered into RGBA16
targets (quantised to k/65535) in the workspace case.

Bars: unshaded frames bit-equal to the FP32 oracle with equal sample
counts; Phong within 1e-4 of it; every frame within 1/255 of the FP64
oracle on rays where FP32 and FP64 take the same discrete decisions."""
import json
import os

import numpy as np
import pytest

import oracle
import voreen_gb300 as v
from voreen_gb300 import synth

from helpers import assert_fp64_parity, oracle_entry_exit, oracle_params

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fixtures")
DENORMALIZING = {v.U8: 255.0, v.U16: 65535.0, v.F32: 1.0}


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _apply_alpha_mode(table, mode):
    """TransFuncBase::applyAlpha (transfuncbase.cpp:177-210): 0 zero alpha,
    1 use alpha, 2 alpha 255 where it is not 0."""
    t = table.copy()
    if mode == 0:
        t[:, 3] = 0
    elif mode == 2:
        t[:, 3] = np.where(t[:, 3] > 0, 255, 0)
    return t


def _load(ctx, name):
    vol = v.Volume.load_vvd(ctx, os.path.join(FIX, name + ".vvd"))
    info = v.read_vvd_header(os.path.join(FIX, name + ".vvd"))
    dt = {v.U8: np.uint8, v.U16: np.uint16, v.F32: np.float32}[info.dtype]
    X, Y, Z = info.dims
    vox = np.fromfile(os.path.join(FIX, name + ".raw"), dt).reshape(Z, Y, X)
    spacing, offset = tuple(info.spacing), tuple(info.offset)
    rwm = (DENORMALIZING[info.dtype], 0.0)
    assert (info.rwm_scale, info.rwm_offset) == rwm  # no RealWorldMapping item in these files
    return vol, vox, spacing, offset, rwm


def _orbit(dims, spacing, offset, az, el, factor=1.6):
    lo, hi = synth.bbox_world(dims, spacing, offset)
    c = [(lo[i] + hi[i]) / 2 for i in range(3)]
    diag = float(np.sqrt(sum((hi[i] - lo[i]) ** 2 for i in range(3))))
    a, e = np.radians(az), np.radians(el)
    pos = (c[0] + factor * diag * np.sin(a) * np.cos(e), c[1] + factor * diag * np.sin(e),
           c[2] + factor * diag * np.cos(a) * np.cos(e))
    return v.make_camera(pos, c, near=0.01 * diag, far=10 * diag)


def _check(ctx, vol, tf, tf_rgba, domain, vox, spacing, offset, rwm, p, label, entry=None, exit_pts=None,
           preint=None):
    if entry is None:
        entry, exit_pts = oracle_entry_exit(vol.desc, p)
    img, st = v.render(ctx, vol, tf, p, entry, exit_pts, v.OUT_RGBA32F)
    ov = oracle.make_volume(vox, spacing, offset, rwm)
    op = oracle_params(p, preint_table=preint)
    g32 = np.zeros(entry.shape[:2], np.uint32)
    g64 = np.zeros(entry.shape[:2], np.uint32)
    o32, s32, fh32 = oracle.render(ov, tf_rgba, domain, op, entry, exit_pts, 32, signature=g32)
    assert st.samples == s32.sum() and s32.sum() > 0
    if p.shading == v.SHADE_NONE:
        np.testing.assert_array_equal(_bits(img), _bits(o32))
    else:
        assert np.abs(img - o32).max() <= 1e-4
    assert (img[..., 3] > 0).mean() > 0.02
    if preint is None:
        o64, s64, fh64 = oracle.render(ov, tf_rgba, domain, op, entry, exit_pts, 64, signature=g64)
        assert_fp64_parity(img, o32, s32, fh32, o64, s64, fh64, p.compositing,
                           1.0 / (max(vox.shape) * p.sampling_rate), shaded=p.shading != v.SHADE_NONE, label=label,
                           sigs=(g32, g64))
    return img


@pytest.mark.parametrize("name", ["nucleon", "walnut"])
@pytest.mark.parametrize("shading", [v.SHADE_NONE, v.SHADE_PHONG])
def test_sample_volume_with_its_tfi(ctx, name, shading):
    vol, vox, spacing, offset, rwm = _load(ctx, name)
    t = v.read_tfi(os.path.join(FIX, name + ".tfi"))
    table = _apply_alpha_mode(v.TransferFunction.bake(t["keys"], t["width"], t["gamma"], t["threshold"]),
                              t["alpha_mode"])
    np.testing.assert_array_equal(table, _apply_alpha_mode(
        oracle.bake_tf(t["keys"], t["width"], t["gamma"], t["threshold"]), t["alpha_mode"]))
    tf = v.TransferFunction(ctx, table, t["domain"])
    p = v.default_params(256, 224)
    p.camera = _orbit(vol.dims, spacing, offset, 35.0, 20.0)
    p.light_position[:] = [*p.camera.position, 1.0]
    p.shading = shading
    _check(ctx, vol, tf, table, t["domain"], vox, spacing, offset, rwm, p,
           f"{name} + {name}.tfi, 256x224, {'Phong' if shading else 'unshaded'}")
    tf.close()
    vol.close()


@pytest.mark.parametrize("shading", [v.SHADE_NONE, v.SHADE_PHONG])
def test_vessel_tree_with_a_preset(ctx, shading):
    """vessel-tree-noisy (101^3 uint8, a .vvd whose raw file is found through
    its path list, an explicit RealWorldMapping of 255) with the "Hot Metal"
    key preset, its domain fitted to the volume's real-world range as
    TransFunc1DKeysProperty::applyDomainFromData does."""
    vol, vox, spacing, offset, rwm = _load(ctx, "vessel-tree-noisy")
    assert vox.shape == (101, 101, 101)
    t = v.read_tfi(os.path.join(FIX, "hot_metal.tfi"))
    domain = (float(vox.min()) * rwm[0] / 255.0, float(vox.max()) * rwm[0] / 255.0)
    width = 256
    table = _apply_alpha_mode(v.TransferFunction.bake(t["keys"], width, t["gamma"], t["threshold"]), t["alpha_mode"])
    np.testing.assert_array_equal(table, _apply_alpha_mode(
        oracle.bake_tf(t["keys"], width, t["gamma"], t["threshold"]), t["alpha_mode"]))
    tf = v.TransferFunction(ctx, table, domain)
    p = v.default_params(240, 200)
    p.camera = _orbit(vol.dims, spacing, offset, -40.0, 30.0)
    p.light_position[:] = [*p.camera.position, 1.0]
    p.shading = shading
    _check(ctx, vol, tf, table, domain, vox, spacing, offset, rwm, p,
           f"vessel-tree-noisy + Hot Metal preset, 240x200, {'Phong' if shading else 'unshaded'}")
    tf.close()
    vol.close()


def test_cpuraycaster_workspace(ctx):
    """cpuraycaster.vws: both CPURaycaster processors of the workspace on
    nucleon with the workspace's camera, canvas, sampling rate and TF --
    classification by the TF, and by the pre-integration table
    ("pre-integrated-approximation": the integral-function table, resolution
    from the TF's bit depth)."""
    case = json.load(open(os.path.join(FIX, "cpuraycaster_vws.json")))
    assert case["volume"] == "nucleon.vvd" and case["proxy"] == "boundingbox"
    vol, vox, spacing, offset, rwm = _load(ctx, "nucleon")
    W, H = case["canvas"]
    cam = case["camera"]
    p = v.default_params(W, H)
    p.camera = v.make_camera(cam["position"], cam["focus"], cam["up"], fovy=cam["fovy"], near=cam["near"],
                             far=cam["far"])
    p.quantize_entry_exit = 1
    entry, exit_pts = oracle_entry_exit(vol.desc, p, quantize=True)
    kinds = {c["classification"]: c for c in case["raycasters"]}
    assert set(kinds) == {"transfer-function", "pre-integrated-approximation"}
    for cls, rc in kinds.items():
        tfd = rc["tf"]
        keys = [(k[0], tuple(k[1]), tuple(k[2])) for k in tfd["keys"]]
        assert len(keys) == 12
        table = _apply_alpha_mode(v.TransferFunction.bake(keys, tfd["width"], tfd["gamma"], tuple(tfd["threshold"])),
                                  tfd["alpha_mode"])
        domain = tuple(tfd["domain"])
        tf = v.TransferFunction(ctx, table, domain)
        q = v.default_params(W, H)
        q.camera, q.quantize_entry_exit, q.sampling_rate = p.camera, 1, rc["sampling_rate"]
        preint = None
        if cls == "pre-integrated-approximation":
            q.classification = v.CLASSIFY_PREINTEGRATED
            res = v.PreIntegrationTable.resolution(tfd["width"], 0)
            src = v.PreIntegrationTable.bake_source(keys, res, tfd["gamma"], tuple(tfd["threshold"]))
            pt = v.PreIntegrationTable(ctx, src, v.sampling_step(vol, q.sampling_rate), True)
            preint = pt.download()
            np.testing.assert_array_equal(_bits(preint), _bits(oracle.preint_table(src, pt.step, True)))
            tf.set_preintegration(pt)
        _check(ctx, vol, tf, table, domain, vox, spacing, offset, rwm, q, f"cpuraycaster.vws {cls}, {W}x{H}",
               entry, exit_pts, preint)
        tf.close()
    vol.close()
