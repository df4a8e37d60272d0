"""Generates the golden vectors in tests/golden from the reference's own code.

Run where the Voreen source tree is available (it is compiled into
oracle/_ref/libvoreen_ref.so by oracle/build.py):

    python tests/golden/make_golden.py [/path/to/voreen]

Outputs (small, committed):
  trilinear.npz  VolumeRAM::getVoxelNormalizedLinear (volumeram.cpp:78-97)
                 on seeded u8 / u16 / f32 volumes with odd dimensions, at
                 random, integer, half-integer and edge positions.
  camera.npz     tgt::mat4::createLookAt / createPerspective
                 (ext/tgt/matrix.h:1196-1247) for seeded cameras.
  iround.npz     tgt::iround (ext/tgt/tgt_math.h:223-225) at values near
                 rounding boundaries.
  tf_bake.npz    the TF bake of TransFunc1D::createTextureData
                 (transfunc1d.cpp:85-103) over the reference's own
                 TransFunc1DKeys::getMappingForValueUByte
                 (1dkeys/transfunc1dkeys.cpp:119-154) and applyGammaToIntensity
                 (oracle/_ref/libvoreen_tf_ref.so) for seeded key sets (split
                 keys, coincident keys, keys on texel values, gamma != 1,
                 thresholds, widths 2..4096) and the keys of the Voreen sample
                 transfer functions nucleon.tfi / walnut.tfi.

    python tests/golden/make_golden.py [/path/to/voreen] [--only tf_bake]
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def trilinear_cases(ref, rng):
    out = {}
    shapes = [(7, 5, 3), (13, 11, 9), (2, 1, 3), (1, 1, 1), (33, 17, 4)]
    for dt_name, dt, code in (("u8", np.uint8, 0), ("u16", np.uint16, 1), ("f32", np.float32, 2)):
        for si, (X, Y, Z) in enumerate(shapes):
            if dt == np.float32:
                vox = rng.random((Z, Y, X), dtype=np.float32)
            else:
                vox = rng.integers(0, np.iinfo(dt).max + 1, size=(Z, Y, X), dtype=dt)
            dims = np.array([X, Y, Z], np.int32)
            n = 400
            pos = rng.uniform(-0.5, 1.0, size=(n, 3)).astype(np.float32) * np.array([X, Y, Z], np.float32)
            # integer, half-integer, edge and just-inside positions
            extra = []
            for i in range(3):
                for v in (0.0, 0.5, X - 1 if i == 0 else (Y - 1 if i == 1 else Z - 1)):
                    p = rng.uniform(0, 1, 3).astype(np.float32) * (dims - 1)
                    p[i] = v
                    extra.append(p)
            extra.append((dims - 1).astype(np.float32))
            extra.append(np.nextafter((dims - 1).astype(np.float32), np.float32(0)))
            pos = np.concatenate([pos, np.array(extra, np.float32)])
            # the march clamps to [0, dim-1] before the lookup
            pos = np.clip(pos, 0, (dims - 1).astype(np.float32)).astype(np.float32)
            res = np.zeros(len(pos), np.float32)
            ref.ref_trilinear(code, _p(vox), dims.ctypes.data_as(C.POINTER(C.c_int)), _p(pos), len(pos), _p(res))
            key = f"{dt_name}_{si}"
            out[key + "_vox"] = vox
            out[key + "_pos"] = pos
            out[key + "_val"] = res
    return out


def camera_cases(ref, rng):
    eyes, foci, ups, look, persp, pp = [], [], [], [], [], []
    for _ in range(24):
        e = rng.uniform(-500, 500, 3).astype(np.float32)
        f = rng.uniform(-50, 50, 3).astype(np.float32)
        u = np.array([0, 1, 0], np.float32) + rng.uniform(-0.3, 0.3, 3).astype(np.float32)
        m = np.zeros(16, np.float32)
        ref.ref_lookat(_p(e), _p(f), _p(u), _p(m))
        eyes.append(e); foci.append(f); ups.append(u); look.append(m)
        fov = np.float32(rng.uniform(0.3, 1.5))
        asp = np.float32(rng.uniform(0.5, 2.5))
        n = np.float32(rng.uniform(0.01, 10))
        fa = np.float32(n + rng.uniform(10, 2000))
        m2 = np.zeros(16, np.float32)
        ref.ref_perspective(fov, asp, n, fa, _p(m2))
        persp.append(m2)
        pp.append([fov, asp, n, fa])
    return {"eye": np.array(eyes), "focus": np.array(foci), "up": np.array(ups), "lookat": np.array(look),
            "persp_params": np.array(pp, np.float32), "persp": np.array(persp)}


def iround_cases(ref, rng):
    base = np.concatenate([np.arange(-4, 5, dtype=np.float32) + np.float32(0.5),
                           rng.uniform(-1000, 1000, 200).astype(np.float32)])
    vals = np.concatenate([base, np.nextafter(base, np.float32(-np.inf)), np.nextafter(base, np.float32(np.inf)),
                           np.array([0.49999997, 1.4999999, 2.5, 4095.5, 254.49998], np.float32)]).astype(np.float32)
    res = np.array([ref.ref_iround(C.c_float(float(v))) for v in vals], np.int32)
    return {"x": vals, "iround": res}


def _random_keys(rng, n):
    xs = np.sort(rng.uniform(0, 1, n)).astype(np.float32)
    keys = []
    for x in xs:
        cl = tuple(int(c) for c in rng.integers(0, 256, 4))
        cr = cl if rng.random() < 0.6 else tuple(int(c) for c in rng.integers(0, 256, 4))
        keys.append((float(x), cl, cr))
    return keys


def _tfi_keys(path):
    """Keys of a Voreen .tfi file (TransFunc1DKeys serialisation): intensity,
    colorL, colorR (= colorL unless split)."""
    import xml.etree.ElementTree as ET
    root = ET.parse(path).getroot()
    keys = []
    for k in root.iter("key"):
        inten = float(k.find("intensity").get("value"))
        split = k.find("split").get("value") in ("true", "1")
        cl = k.find("colorL")
        cl = tuple(int(cl.get(c)) for c in "rgba")
        cr = k.find("colorR") if split else None
        cr = tuple(int(cr.get(c)) for c in "rgba") if cr is not None else cl
        keys.append((inten, cl, cr))
    return keys


def tf_bake_cases(rng, reference_root):
    cases = []
    for i in range(40):
        keys = _random_keys(rng, int(rng.integers(1, 12)))
        width = int(rng.choice([2, 3, 256, 1000, 4096]))
        gamma = 1.0 if i % 3 else float(rng.uniform(0.3, 3.0))
        thr = (0.0, 1.0) if i % 4 else (float(rng.uniform(0, 0.3)), float(rng.uniform(0.6, 1.0)))
        cases.append((keys, width, gamma, thr))
    # keys exactly on texel values, coincident keys, descending ramps, one key, none
    on = [float(np.float32(k) / np.float32(255)) for k in (0, 40, 41, 128, 200, 255)]
    cases.append(([(on[0], (0, 0, 255, 0)), (on[1], (0, 0, 255, 0)), (on[2], (9, 9, 250, 3)),
                   (on[3], (250, 10, 10, 200)), (on[4], (30, 200, 30, 255), (200, 30, 30, 0)),
                   (on[5], (255, 255, 255, 255))], 256, 1.0, (0.0, 1.0)))
    cases.append(([(0.25, (255, 0, 0, 255)), (0.25, (0, 255, 0, 10)), (0.75, (0, 0, 255, 128)),
                   (0.75, (255, 255, 0, 64), (1, 2, 3, 4))], 4096, 1.0, (0.0, 1.0)))
    cases.append(([(0.0, (255, 255, 255, 255)), (1.0, (0, 0, 0, 0))], 1000, 0.5, (0.2, 0.9)))
    cases.append(([(0.6, (10, 20, 30, 40), (50, 60, 70, 80))], 256, 2.0, (0.0, 1.0)))
    cases.append(([], 64, 1.0, (0.0, 1.0)))
    tfdir = os.path.join(reference_root, "resource", "voreencore", "transferfuncs")
    for name in ("nucleon.tfi", "walnut.tfi"):
        keys = _tfi_keys(os.path.join(tfdir, name))
        for width in (256, 4096):
            cases.append((keys, width, 1.0, (0.0, 1.0)))
    out = {"n": np.array(len(cases))}
    for i, (keys, width, gamma, thr) in enumerate(cases):
        table = oracle.ref_bake_tf(keys, width, gamma, thr, reference_root)
        out[f"c{i}_intensity"] = np.array([k[0] for k in keys], np.float32)
        out[f"c{i}_colors"] = np.array([list(k[1]) + list(k[2] if len(k) > 2 else k[1]) for k in keys],
                                       np.uint8).reshape(-1, 8)
        out[f"c{i}_params"] = np.array([width, gamma, thr[0], thr[1]], np.float64)
        out[f"c{i}_table"] = table
    return out


def main(reference_root=None, only=None):
    from oracle import build as obuild
    reference_root = reference_root or obuild.DEFAULT_REFERENCE
    if only == "tf_bake":
        if oracle.ref_tf_lib(reference_root) is None:
            raise SystemExit("reference sources not found: cannot build oracle/_ref")
        np.savez_compressed(os.path.join(HERE, "tf_bake.npz"),
                            **tf_bake_cases(np.random.default_rng(20261204), reference_root))
        print("tf_bake.npz written to", HERE)
        return
    ref = oracle.ref_lib(reference_root)
    if ref is None:
        raise SystemExit("reference sources not found: cannot build oracle/_ref")
    rng = np.random.default_rng(20261203)
    np.savez_compressed(os.path.join(HERE, "trilinear.npz"), **trilinear_cases(ref, rng))
    np.savez_compressed(os.path.join(HERE, "camera.npz"), **camera_cases(ref, rng))
    np.savez_compressed(os.path.join(HERE, "iround.npz"), **iround_cases(ref, rng))
    np.savez_compressed(os.path.join(HERE, "tf_bake.npz"),
                        **tf_bake_cases(np.random.default_rng(20261204), reference_root))
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("reference_root", nargs="?", default=None)
    ap.add_argument("--only", choices=["tf_bake"], default=None)
    a = ap.parse_args()
    main(a.reference_root, a.only)
