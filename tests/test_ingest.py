"""Volume ingest (.vvd) header parsing on the CPU: synthetic files in both
RawData forms, Voreen's defaults, error statuses, and -- where the Voreen tree
is present -- the sample volumes it ships, checked against an independent
XML parse and their own VolumeMinMax derived items."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import voreen_gb300 as v
from voreen_gb300 import _abi

from oracle import build as _obuild

REF_VOLUMES = os.path.join(_obuild.DEFAULT_REFERENCE, "resource", "voreenve", "volumes")


def test_synthetic_headers(vrc_lib, tmp_path):
    vox = (np.arange(5 * 6 * 7) % 251).astype(np.uint8).reshape(5, 6, 7)
    v.write_vvd(str(tmp_path / "a.vvd"), vox, spacing=(0.5, 0.25, 2.0), offset=(-1.0, 0.5, 3.0), rwm=(255.0, -1.5))
    i = v.read_vvd_header(str(tmp_path / "a.vvd"))
    assert (i.dtype, tuple(i.dims)) == (v.U8, (7, 6, 5))
    assert tuple(i.spacing) == (0.5, 0.25, 2.0) and tuple(i.offset) == (-1.0, 0.5, 3.0)
    assert (i.rwm_scale, i.rwm_offset, i.has_minmax) == (255.0, -1.5, 0)
    assert i.raw_path.decode() == str(tmp_path / "a.raw")
    # path-list form: the first existing entry is taken; defaults for absent meta items
    v.write_vvd(str(tmp_path / "b.vvd"), vox.astype(np.uint16), path_list=True)
    (tmp_path / "b.vvd").write_text((tmp_path / "b.vvd").read_text().replace(
        '<MetaItem name="Offset"', '<MetaItem name="Ignored"').replace('<MetaItem name="Spacing"', '<MetaItem name="X"'))
    i = v.read_vvd_header(str(tmp_path / "b.vvd"))
    assert i.dtype == v.U16 and tuple(i.spacing) == (1.0, 1.0, 1.0) and tuple(i.offset) == (0.0, 0.0, 0.0)
    # no RealWorldMapping item: the denormalizing mapping of the format, as
    # VvdVolumeReader sets it (vvdvolumereader.cpp:102-120)
    assert (i.rwm_scale, i.rwm_offset) == (65535.0, 0.0)
    for dt, scale in ((np.uint8, 255.0), (np.float32, 1.0)):
        v.write_vvd(str(tmp_path / "d.vvd"), vox.astype(dt))
        j = v.read_vvd_header(str(tmp_path / "d.vvd"))
        assert (j.rwm_scale, j.rwm_offset) == (scale, 0.0)
    assert i.raw_path.decode() == str(tmp_path / "b.raw")


def test_header_errors(vrc_lib, tmp_path):
    vox = np.zeros((2, 3, 4), np.float32)
    v.write_vvd(str(tmp_path / "c.vvd"), vox)
    text = (tmp_path / "c.vvd").read_text()
    (tmp_path / "d.vvd").write_text(text.replace('format="float"', 'format="int16"'))
    info = _abi.VvdInfo()
    L = v.lib()
    assert L.vrc_vvd_read_header(str(tmp_path / "d.vvd").encode(), info) == 4      # VRC_ERR_UNSUPPORTED
    os.remove(tmp_path / "c.raw")
    assert L.vrc_vvd_read_header(str(tmp_path / "c.vvd").encode(), info) == 0      # header alone parses
    (tmp_path / "e.vvd").write_text(text.replace('filename="c.raw"', ''))
    assert L.vrc_vvd_read_header(str(tmp_path / "e.vvd").encode(), info) == 6      # no raw file: not ready
    assert L.vrc_vvd_read_header(str(tmp_path / "none.vvd").encode(), info) == 6


def _ref_files():
    if not os.path.isdir(REF_VOLUMES):
        return []
    return sorted(f for f in os.listdir(REF_VOLUMES) if f.endswith(".vvd"))


@pytest.mark.parametrize("name", _ref_files() or ["(no Voreen tree)"])
def test_shipped_volumes(vrc_lib, name):
    if name == "(no Voreen tree)":
        pytest.skip("the Voreen tree with its sample volumes is not present")
    path = os.path.join(REF_VOLUMES, name)
    text = open(path, encoding="utf-8").read()
    root = ET.fromstring(text[text.index("<?xml"):])  # some files open with a comment before the declaration
    raw = root.find(".//RawData")
    info = _abi.VvdInfo()
    st = v.lib().vrc_vvd_read_header(path.encode(), info)
    fmt = raw.get("format")
    if fmt not in ("uint8", "uint16", "float"):
        assert st == 4  # multi-channel data: not a scalar volume
        return
    assert st == 0
    assert tuple(info.dims) == tuple(int(raw.get(k)) for k in "xyz")
    assert info.dtype == {"uint8": v.U8, "uint16": v.U16, "float": v.F32}[fmt]
    for key, field in (("Spacing", info.spacing), ("Offset", info.offset)):
        item = root.find(f".//MetaItem[@name='{key}']/value")
        if item is not None:
            assert tuple(field) == tuple(np.float32(item.get(k)) for k in "xyz")
    rwm = root.find(".//MetaItem[@name='RealWorldMapping']/value")
    if rwm is not None:
        assert (info.rwm_scale, info.rwm_offset) == (np.float32(rwm.get("scale")), np.float32(rwm.get("offset")))
    else:
        assert (info.rwm_scale, info.rwm_offset) == ({"uint8": 255.0, "uint16": 65535.0, "float": 1.0}[fmt], 0.0)
    # Voreen's own VolumeMinMax against the raw voxels normalised as vrc normalises them
    mm = root.find(".//DerivedItem[@type='VolumeMinMax']")
    if mm is not None and os.path.exists(info.raw_path.decode()):
        if mm.get("minNorm") is not None:
            lo, hi = float(mm.get("minNorm")), float(mm.get("maxNorm"))
        else:
            lo = float(mm.find("minNormValues/channel").get("value"))
            hi = float(mm.find("maxNormValues/channel").get("value"))
        assert info.has_minmax == 1 and (info.min_norm, info.max_norm) == (np.float32(lo), np.float32(hi))
        vox = np.fromfile(info.raw_path.decode(), {v.U8: np.uint8, v.U16: np.uint16, v.F32: np.float32}[info.dtype])
        scale = {v.U8: 255.0, v.U16: 65535.0, v.F32: 1.0}[info.dtype]
        assert np.float32(vox.min() / scale) == pytest.approx(lo, abs=1e-7)
        assert np.float32(vox.max() / scale) == pytest.approx(hi, abs=1e-7)


REF_TFS = os.path.join(os.path.dirname(REF_VOLUMES), "..", "voreencore", "transferfuncs")

TFI = """<?xml version="1.0" ?>
<VoreenData version="1">
    <TransFuncIntensity type="TransFuncIntensity">
        <texDimensions x="4096" y="1" z="1" />
        <gammaValue value="1.5" />
        <domain x="-100" y="3000.5" />
        <Keys>
            <key type="TransFuncMappingKey">
                <intensity value="0.25" />
                <split value="false" />
                <colorL r="10" g="20" b="30" a="40" />
            </key>
            <key type="TransFuncMappingKey">
                <intensity value="0.5" />
                <split value="true" />
                <colorL r="1" g="2" b="3" a="4" />
                <colorR r="250" g="240" b="230" a="220" />
            </key>
        </Keys>
    </TransFuncIntensity>
</VoreenData>
"""


def test_read_tfi_fields_defaults_and_split_keys(vrc_lib, tmp_path):
    f = tmp_path / "t.tfi"
    f.write_text(TFI)
    t = v.read_tfi(str(f))
    assert t["width"] == 4096 and t["gamma"] == 1.5 and t["alpha_mode"] == 1  # alphaMode absent: 1
    assert t["domain"] == (-100.0, 3000.5) and t["threshold"] == (0.0, 1.0)  # threshold absent: (0, 1)
    assert t["keys"] == [(0.25, (10, 20, 30, 40), (10, 20, 30, 40)), (0.5, (1, 2, 3, 4), (250, 240, 230, 220))]
    # the keys bake like keys given directly
    a = v.TransferFunction.bake([(k[0], k[1], k[2]) for k in t["keys"]], 256, t["gamma"], t["threshold"])
    b = v.TransferFunction.bake([(0.25, (10, 20, 30, 40)), (0.5, (1, 2, 3, 4), (250, 240, 230, 220))], 256, 1.5)
    np.testing.assert_array_equal(a, b)
    with pytest.raises(v.VrcError):
        v.read_tfi(str(tmp_path / "missing.tfi"))
    (tmp_path / "bad.tfi").write_text("<VoreenData><SomethingElse/></VoreenData>")
    with pytest.raises(v.VrcError):
        v.read_tfi(str(tmp_path / "bad.tfi"))


def test_processor_loads_tfi(vrc_lib, tmp_path):
    from voreen_gb300.raycaster import CudaRaycaster
    f = tmp_path / "t.tfi"
    f.write_text(TFI)
    r = CudaRaycaster()
    r.load_transfer_function(str(f))
    assert r.transferFunction.domain == (-100.0, 3000.5) and r.transferFunction.domain_fitted
    assert r.transferFunction.gamma == 1.5 and len(r.transferFunction.keys) == 2
    r.close()


def _etree_tfi(path):
    root = ET.parse(path).getroot().find("TransFuncIntensity")
    def xy(tag, default):
        e = root.find(tag)
        return (float(e.get("x")), float(e.get("y"))) if e is not None else default
    keys = []
    for k in root.find("Keys").findall("key"):
        col = lambda e: tuple(int(e.get(c)) for c in "rgba")
        cl = col(k.find("colorL"))
        split = k.find("split").get("value") == "true"
        keys.append((float(np.float32(float(k.find("intensity").get("value")))), cl,
                     col(k.find("colorR")) if split else cl))
    g = root.find("gammaValue")
    return {"keys": keys, "domain": xy("domain", (0.0, 1.0)), "threshold": xy("threshold", (0.0, 1.0)),
            "gamma": float(g.get("value")) if g is not None else 1.0}


@pytest.mark.skipif(not os.path.isdir(REF_TFS), reason="the Voreen source tree is not present")
def test_reference_tfi_files_equal_an_independent_parse(vrc_lib):
    """The reference's own .tfi files (sample and preset transfer functions)
    read as Python's XML parser reads them."""
    paths = [os.path.join(REF_TFS, f) for f in ("nucleon.tfi", "walnut.tfi")]
    pre = os.path.join(REF_TFS, "presets", "1dkeys")
    if os.path.isdir(pre):
        paths += sorted(os.path.join(pre, f) for f in os.listdir(pre) if f.endswith(".tfi"))
    assert len(paths) >= 2
    for p in paths:
        t, ref = v.read_tfi(p), _etree_tfi(p)
        assert t["keys"] == ref["keys"], p
        assert t["domain"] == tuple(np.float32(ref["domain"]).tolist()), p
        assert t["threshold"] == tuple(np.float32(ref["threshold"]).tolist()), p
        assert t["gamma"] == float(np.float32(ref["gamma"])), p
