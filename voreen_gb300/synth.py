"""Seeded workloads: procedural volumes, transfer functions and orbit cameras.

These are the benchmark configurations of the raycaster (restated as seeded
synthetic inputs; no dataset is involved) and the generator of the learned
upsampler's training renders. Config k with seed s uses generator seed
1000 * k + s.
"""
from __future__ import annotations

import math
import random
from dataclasses import dataclass, field

import numpy as np

from . import (DVR, MIP, SHADE_NONE, SHADE_PHONG, U8, U16, F32, default_params, make_camera, synth_volume)

BLOBS, SHELLS = 0, 1


@dataclass
class Workload:
    name: str
    voxels: np.ndarray              # (Z, Y, X)
    spacing: tuple
    tf_keys: list
    tf_width: int
    domain: tuple                   # TF domain in real-world units
    width: int
    height: int
    sampling_rate: float
    compositing: int = DVR
    shading: int = SHADE_NONE
    camera_pos: tuple = (0.0, 0.0, 3.0)
    camera_focus: tuple = (0.0, 0.0, 0.0)
    fovy: float = 45.0
    near: float = 0.1
    far: float = 50.0
    light_pos: tuple = (2.3, 1.5, 1.5, 1.0)
    extra: dict = field(default_factory=dict)

    @property
    def dims(self):
        return (self.voxels.shape[2], self.voxels.shape[1], self.voxels.shape[0])

    def params(self, **over):
        p = default_params(self.width, self.height)
        p.sampling_rate = self.sampling_rate
        p.compositing = self.compositing
        p.shading = self.shading
        p.light_position[:] = list(self.light_pos)
        p.camera = make_camera(self.camera_pos, self.camera_focus, fovy=self.fovy, near=self.near, far=self.far)
        for k, v in over.items():
            setattr(p, k, v)
        return p


def bbox_world(dims, spacing, offset=(0.0, 0.0, 0.0)):
    lo = [offset[i] - 0.5 * spacing[i] for i in range(3)]
    hi = [offset[i] + (dims[i] - 0.5) * spacing[i] for i in range(3)]
    return lo, hi


def orbit_camera(dims, spacing, azimuth_deg: float, elevation_deg: float, dist_factor: float = 2.5):
    """Perspective orbit around the world bounding box centre at
    dist_factor x the box diagonal; near/far enclose the box."""
    lo, hi = bbox_world(dims, spacing)
    c = [(lo[i] + hi[i]) / 2 for i in range(3)]
    diag = math.sqrt(sum((hi[i] - lo[i]) ** 2 for i in range(3)))
    dist = dist_factor * diag
    az, el = math.radians(azimuth_deg), math.radians(elevation_deg)
    pos = (c[0] + dist * math.sin(az) * math.cos(el), c[1] + dist * math.sin(el), c[2] + dist * math.cos(az) * math.cos(el))
    return pos, tuple(c), max(1e-3, dist - diag), dist + diag


def tf_keys_c1():
    """256-entry ramp: alpha 0 below intensity 40/255, linear to 0.6 at 1;
    colour blue -> red."""
    t = 40.0 / 255.0
    mix = lambda a: (int(round(255 * a)), 0, int(round(255 * (1 - a))))
    return [(0.0, (*mix(0.0), 0)), (t, (*mix(t), 0)), (1.0, (*mix(1.0), 153))]


def tf_keys_trapezoids(centers, seed: int, alpha_range=(0.1, 0.8), top=(0.004, 0.015), ramp=(0.006, 0.02)):
    """One trapezoid per centre (TF coordinates in [0,1]), random widths,
    opacity and colour; keys sorted, trapezoids kept apart."""
    rng = random.Random(seed)
    keys = []
    for c in sorted(centers):
        h_top = rng.uniform(*top)
        h_ramp = rng.uniform(*ramp)
        a = int(round(255 * rng.uniform(*alpha_range)))
        col = tuple(int(rng.uniform(60, 255)) for _ in range(3))
        pts = [c - h_top - h_ramp, c - h_top, c + h_top, c + h_top + h_ramp]
        pts = [min(1.0, max(0.0, p)) for p in pts]
        keys += [(pts[0], (*col, 0)), (pts[1], (*col, a)), (pts[2], (*col, a)), (pts[3], (*col, 0))]
    # keep keys strictly ordered
    out = []
    for k in keys:
        if out and k[0] <= out[-1][0]:
            k = (min(1.0, out[-1][0] + 1e-6), k[1])
        out.append(k)
    return out


def config1(seed: int = 1, size=(128, 128, 128), image=(512, 512), azimuth=30.0, elevation=20.0,
            volume_fn=None) -> Workload:
    """Plain DVR, 128^3 u8 Gaussian blobs, 256-entry ramp TF, 512^2, rate 2.
    volume_fn: the generator (kind, dtype, dims, seed) -> voxels, by default
    the library's vrc_synth_volume."""
    vox = (volume_fn or synth_volume)(BLOBS, U8, size, 1000 * 1 + seed)
    pos, focus, near, far = orbit_camera(size, (1, 1, 1), azimuth, elevation)
    return Workload("plain DVR 128^3 u8 512x512", vox, (1.0, 1.0, 1.0), tf_keys_c1(), 256, (0.0, 1.0), image[0],
                    image[1], 2.0, DVR, SHADE_NONE, pos, focus, near=near, far=far)


SHELL_INTENSITIES = (200, 1000, 1800, 2600, 3200, 4000)


def shells_tf(vox_u16: np.ndarray, seed: int, n_peaks: int = 5, rwm=(1.0, 0.0)):
    """4096-entry TF with trapezoids on n_peaks of the shell intensities, and
    the domain fitted to the volume's real-world [min, max]."""
    mn = float(vox_u16.min()) / 65535.0
    mx = float(vox_u16.max()) / 65535.0
    lo, hi = mn * rwm[0] + rwm[1], mx * rwm[0] + rwm[1]
    rng = random.Random(seed)
    chosen = sorted(rng.sample(SHELL_INTENSITIES, n_peaks))
    centers = [((c / 65535.0 * rwm[0] + rwm[1]) - lo) / (hi - lo) for c in chosen]
    return tf_keys_trapezoids(centers, seed + 7), (lo, hi)


def config2(seed: int = 1, size=(512, 512, 512), image=(1920, 1080), compositing=DVR, azimuth=35.0,
            elevation=25.0, dist_factor=1.25, volume_fn=None) -> Workload:
    """CT-like shaded DVR (or MIP): 512^3 u16 nested shells, spacing
    (0.7, 0.7, 1.0), 4096-entry 5-trapezoid TF, Phong, 1920x1080, rate 2.
    The light sits at the camera position; the camera orbits at 1.25 x the box
    diagonal so the volume fills most of the frame. volume_fn as in config1."""
    vox = (volume_fn or synth_volume)(SHELLS, U16, size, 1000 * 2 + seed)
    spacing = (0.7, 0.7, 1.0)
    keys, domain = shells_tf(vox, 1000 * 2 + seed)
    pos, focus, near, far = orbit_camera(size, spacing, azimuth, elevation, dist_factor)
    shading = SHADE_PHONG if compositing == DVR else SHADE_NONE
    return Workload(f"CT-like {'shaded DVR' if compositing == DVR else 'MIP'} {size[0]}x{size[1]}x{size[2]} u16 "
                    f"{image[0]}x{image[1]}", vox, spacing, keys, 4096, domain, image[0], image[1], 2.0,
                    compositing, shading, pos, focus, near=near, far=far, light_pos=(*pos, 1.0))


BATCH_DIMS = ((64, 64, 64), (128, 128, 128), (256, 256, 256), (384, 256, 200), (512, 512, 512))
BATCH_IMAGES = ((256, 256), (512, 512), (1024, 1024), (1920, 1080), (2048, 2048))
BATCH_DTYPES = (U8, U16, F32)


def random_trapezoid_keys(rng: random.Random, n: int = 3):
    """n trapezoids at random TF positions in [0.15, 0.95], kept apart."""
    slots = sorted(rng.sample(range(n * 3), n))
    centers = [0.15 + (0.8 * (sl + rng.uniform(0.3, 0.7))) / (n * 3) for sl in slots]
    return tf_keys_trapezoids(centers, rng.randrange(1 << 30), alpha_range=(0.15, 0.7), top=(0.01, 0.03),
                              ramp=(0.01, 0.03))


def config3(seed: int = 1, n: int = 64, dims_set=BATCH_DIMS, images=BATCH_IMAGES, dtypes=BATCH_DTYPES):
    """Batched requests: volume sizes from dims_set with mixed dtypes
    (blobs or shells), image sizes from `images`, random orbit cameras and
    random 256- or 4096-entry 3-trapezoid TFs, DVR + Phong. Volumes are
    shared between requests of the same (size, dtype, content). Returns
    (volumes: {key: (voxels, spacing)}, requests: [dict])."""
    rng = random.Random(3000 + seed)
    volumes, requests = {}, []
    for i in range(n):
        dims = rng.choice(dims_set)
        dt = rng.choice(dtypes)
        kind = rng.choice((BLOBS, SHELLS))
        key = (dims, dt, kind)
        if key not in volumes:
            volumes[key] = (synth_volume(kind, dt, dims, 3000 + seed * 100 + len(volumes)), (1.0, 1.0, 1.0))
        W, H = rng.choice(images)
        pos, focus, near, far = orbit_camera(dims, (1.0, 1.0, 1.0), rng.uniform(0, 360), rng.uniform(-60, 60),
                                             rng.uniform(1.1, 2.0))
        requests.append({"volume": key, "width": W, "height": H, "camera": (pos, focus, near, far),
                         "tf_width": rng.choice((256, 4096)), "tf_keys": random_trapezoid_keys(rng),
                         "light": (*pos, 1.0)})
    return volumes, requests


def tubes_tf(seed: int, n_peaks: int = 2, domain=(0.0, 4095.0 / 65535.0)):
    """4096-entry TF with n_peaks trapezoids inside the tube intensity range
    (1500..4000 of 4095) for a volume whose real-world domain is `domain`."""
    rng = random.Random(seed)
    lo, hi = domain
    centers = []
    for k in range(n_peaks):
        raw = rng.uniform(1600 + k * 2400 / n_peaks, 1600 + (k + 1) * 2400 / n_peaks - 200)
        centers.append((raw / 65535.0 - lo) / (hi - lo))
    return tf_keys_trapezoids(centers, seed + 3, alpha_range=(0.2, 0.7), top=(0.01, 0.03), ramp=(0.02, 0.05)), domain
