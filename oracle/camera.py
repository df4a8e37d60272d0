"""Camera matrices for the oracle side -- TEST INFRASTRUCTURE ONLY.

FP64 numpy restatement of the reference's camera chain, so that the oracle
(and the benchmark's CPU arm) computes entry/exit points without the
product library:
  * view: tgt::Matrix4::createLookAt (ext/tgt/matrix.h:1196-1209);
  * projection: tgt::Camera::getProjectionMatrix for PERSPECTIVE
    (ext/tgt/camera.cpp:196-205) over Matrix4::createPerspective
    (ext/tgt/matrix.h:1229-1247), fovy clamped to [6, 175] degrees and
    widened for windows taller than wide;
  * textureToWorld = voxelToPhysical * textureToVoxel with physicalToWorld
    the identity (src/core/datastructures/volume/volumebase.cpp:194-229).
Pinned against tests/golden/camera.npz (outputs of the reference's own
createLookAt / createPerspective).
"""
from __future__ import annotations

import math

import numpy as np


def _norm(v):
    n = math.sqrt(float(v[0]) ** 2 + float(v[1]) ** 2 + float(v[2]) ** 2)
    return v / n if n > 0 else v


def look_at(eye, focus, up) -> np.ndarray:
    e = np.asarray(eye, np.float64)
    look = _norm(np.asarray(focus, np.float64) - e)
    u = _norm(np.asarray(up, np.float64))
    strafe = _norm(np.cross(look, u))
    up2 = np.cross(strafe, look)
    r = np.eye(4)
    r[0, :3], r[1, :3], r[2, :3] = strafe, up2, -look
    t = np.eye(4)
    t[:3, 3] = -e
    return r @ t


def perspective(fovy_deg: float, near: float, far: float, window_ratio: float, frustum_ratio: float = 1.0):
    fovy = min(max(float(fovy_deg), 6.0), 175.0)
    ratio = frustum_ratio if frustum_ratio > 0 else 1.0
    deg = math.pi / 180.0
    fov = fovy * deg
    if window_ratio < 1.0:
        fov = math.atan(math.tan(fovy * deg / 2.0) / (window_ratio * ratio)) * 2.0
    aspect = ratio * window_ratio
    f = 1.0 / math.tan(fov / 2.0)
    n, fa = float(near), float(far)
    r = np.zeros((4, 4))
    r[0, 0] = f / aspect
    r[1, 1] = f
    r[2, 2] = (n + fa) / (n - fa)
    r[2, 3] = (2.0 * fa * n) / (n - fa)
    r[3, 2] = -1.0
    return r


def texture_to_world(dims, spacing, offset=(0.0, 0.0, 0.0)) -> np.ndarray:
    r = np.eye(4)
    for i in range(3):
        r[i, i] = float(np.float32(spacing[i])) * dims[i]
        r[i, 3] = float(np.float32(offset[i])) - 0.5 * float(np.float32(spacing[i]))
    return r


def inverse_mvp(position, focus, up, fovy_deg, near, far, width, height, dims, spacing, offset=(0.0, 0.0, 0.0),
                frustum_ratio=1.0) -> np.ndarray:
    """inverse(projection * view * textureToWorld), row-major 4 x 4 FP64,
    for a width x height image. Camera values are taken as the float32 the
    renderer stores them in."""
    f32 = lambda xs: [float(np.float32(x)) for x in xs]
    V = look_at(f32(position), f32(focus), f32(up))
    P = perspective(float(np.float32(fovy_deg)), float(np.float32(near)), float(np.float32(far)),
                    width / height, float(np.float32(frustum_ratio)))
    return np.linalg.inv(P @ V @ texture_to_world(dims, spacing, offset))
