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


def main(reference_root=None):
    ref = oracle.ref_lib(reference_root)
    if ref is None:
        raise SystemExit("reference sources not found: cannot build oracle/_ref")
    rng = np.random.default_rng(20261203)
    np.savez_compressed(os.path.join(HERE, "trilinear.npz"), **trilinear_cases(ref, rng))
    np.savez_compressed(os.path.join(HERE, "camera.npz"), **camera_cases(ref, rng))
    np.savez_compressed(os.path.join(HERE, "iround.npz"), **iround_cases(ref, rng))
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
