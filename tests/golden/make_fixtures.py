"""Copies the reference's own fixed-input cases into tests/golden/fixtures,
so that the GPU tests can render them where the Voreen tree is absent.

Run where the Voreen source tree is available:

    python tests/golden/make_fixtures.py [/path/to/voreen]

Copied unchanged (data files, not code):
  resource/voreenve/volumes/nucleon.{vvd,raw}   41^3 uint8
  resource/voreenve/volumes/walnut.{vvd,raw}    128x96x114 uint16
  resource/voreenve/volumes/vessel-tree-noisy.{vvd,raw}   101^3 uint8 (path list, RealWorldMapping 255)
  resource/voreencore/transferfuncs/{nucleon,walnut}.tfi
  resource/voreencore/transferfuncs/presets/1dkeys/101_Hot Metal.tfi -> hot_metal.tfi
Extracted from modules/base/test/render/cpuraycaster.vws (the reference's
CPURaycaster regression workspace) into cpuraycaster_vws.json: the canvas
size, the MeshEntryExitPoints camera, the proxy mode and, per CPURaycaster
processor, its classification, sampling rate and 1D transfer function
(keys, texture width, domain, threshold, gamma, alpha mode).
"""
from __future__ import annotations

import json
import os
import shutil
import sys
import xml.etree.ElementTree as ET

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "fixtures")


def _keys(tf):
    keys = []
    for k in tf.iter("key"):
        inten = float(k.get("intensity") if k.get("intensity") is not None else k.find("intensity").get("value"))
        split = (k.get("split") or (k.find("split").get("value") if k.find("split") is not None else "false"))
        cl = k.find("colorL")
        cl = [int(cl.get(c)) for c in "rgba"]
        cr = k.find("colorR")
        cr = [int(cr.get(c)) for c in "rgba"] if split in ("true", "1") and cr is not None else cl
        keys.append([inten, cl, cr])
    return keys


def workspace_case(vws_path):
    root = ET.parse(vws_path).getroot()
    procs = {p.get("name"): p for p in root.iter("Processor") if p.get("type") is not None and p.get("name")}

    def prop(p, key):
        for q in p.iter("Property"):
            if q.get("mapKey") == key:
                return q
        return None

    canvas = prop(procs["Canvas"], "canvasSize").find("value")
    cam = prop(procs["MeshEntryExitPoints"], "camera")
    vec = lambda e: [float(e.get(c)) for c in "xyz"]
    camera = {"position": vec(cam.find("position")), "focus": vec(cam.find("focus")),
              "up": vec(cam.find("upVector")), "fovy": float(cam.get("fovy")), "near": float(cam.get("frustNear")),
              "far": float(cam.get("frustFar")), "projection_mode": int(cam.get("projectionMode"))}
    casters = []
    for name, p in procs.items():
        if p.get("type") != "CPURaycaster":
            continue
        tfp = prop(p, "tFunc1DKeys").find("TransferFunction")
        casters.append({
            "name": name,
            "classification": prop(p, "classification").get("value"),
            "sampling_rate": float(prop(p, "samplingRate").get("value")),
            "tf": {"width": int(tfp.find("texDimensions").get("x")),
                   "domain": [float(tfp.find("domain").get(c)) for c in "xy"],
                   "threshold": [float(tfp.find("threshold").get(c)) for c in "xy"],
                   "gamma": float(tfp.get("gammaValue", "1")), "alpha_mode": int(tfp.get("alphaMode", "1")),
                   "keys": _keys(tfp)}})
    proxy = prop(procs["OptimizedProxyGeometry"], "modeString").get("value")
    vol = prop(procs["VolumeSource"], "volumeURL").get("url")
    return {"source": "modules/base/test/render/cpuraycaster.vws", "volume": os.path.basename(vol),
            "canvas": [int(canvas.get("x")), int(canvas.get("y"))], "camera": camera, "proxy": proxy,
            "raycasters": sorted(casters, key=lambda c: c["name"])}


def main(reference_root=None):
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import build as obuild
    root = reference_root or obuild.DEFAULT_REFERENCE
    vols = os.path.join(root, "resource", "voreenve", "volumes")
    tfs = os.path.join(root, "resource", "voreencore", "transferfuncs")
    if not os.path.isdir(vols):
        raise SystemExit(f"Voreen tree not found at {root}")
    os.makedirs(OUT, exist_ok=True)
    for name in ("nucleon.vvd", "nucleon.raw", "walnut.vvd", "walnut.raw", "vessel-tree-noisy.vvd",
                 "vessel-tree-noisy.raw"):
        shutil.copyfile(os.path.join(vols, name), os.path.join(OUT, name))
    for name in ("nucleon.tfi", "walnut.tfi"):
        shutil.copyfile(os.path.join(tfs, name), os.path.join(OUT, name))
    shutil.copyfile(os.path.join(tfs, "presets", "1dkeys", "101_Hot Metal.tfi"), os.path.join(OUT, "hot_metal.tfi"))
    case = workspace_case(os.path.join(root, "modules", "base", "test", "render", "cpuraycaster.vws"))
    with open(os.path.join(OUT, "cpuraycaster_vws.json"), "w") as f:
        json.dump(case, f, indent=1)
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
