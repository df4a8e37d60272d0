"""Seeded random parity sweep: volume shape and dtype, brick and skip-cell
size, real-world mapping, TF keys, camera, sampling rate and compositing mode
drawn at random per case; every unshaded image must equal the FP32 oracle
bit for bit with the same sample counts, shaded ones within 1e-4."""
import numpy as np
import pytest

import voreen_gb300 as v

from helpers import Case, assert_fp64_parity

pytestmark = pytest.mark.gpu

MODES = [v.DVR, v.MIP, v.ISO, v.MOP, v.MIDA, v.FHP]


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _volume(rng, dims, dtype):
    """A few Gaussian blobs plus noise on a (Z, Y, X) grid, in the dtype's range."""
    X, Y, Z = dims
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    f = np.zeros((Z, Y, X), np.float64)
    for _ in range(int(rng.integers(1, 5))):
        c = rng.uniform(0, 1, 3) * np.array([X, Y, Z])
        s = rng.uniform(1.0, 0.4 * max(dims) + 1.0)
        f += rng.uniform(0.3, 1.0) * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    f += rng.uniform(0, 0.05, f.shape)
    f = np.clip(f, 0, 1)
    if dtype == np.float32:
        return (f * 2.0 - 0.5).astype(np.float32)
    return np.floor(f * np.iinfo(dtype).max).astype(dtype)


def _keys(rng):
    n = int(rng.integers(2, 7))
    pos = np.sort(rng.uniform(0, 1, n))
    pos[0], pos[-1] = 0.0, 1.0
    keys = []
    for p in pos:
        a = 0 if rng.uniform() < 0.35 else int(rng.integers(1, 256))
        keys.append((float(p), tuple(int(c) for c in rng.integers(0, 256, 3)) + (a,)))
    return keys


@pytest.mark.parametrize("seed", range(64))
def test_random_case_matches_oracle(ctx, seed):
    rng = np.random.default_rng(7000 + seed)
    dims = tuple(int(d) for d in rng.integers(1, 44, size=3))
    dtype = [np.uint8, np.uint16, np.float32][int(rng.integers(0, 3))]
    vox = _volume(rng, dims, dtype)
    rwm = (1.0, 0.0) if dtype != np.float32 else (float(rng.choice([-1.0, 1.0]) * rng.uniform(0.5, 2.0)),
                                                   float(rng.uniform(-0.5, 0.5)))
    norm = vox.astype(np.float64) / (1.0 if dtype == np.float32 else np.iinfo(dtype).max)
    rw = norm * rwm[0] + rwm[1]
    domain = (float(rw.min()), float(rw.max())) if rng.uniform() < 0.7 else (0.0, 1.0)
    width = 256 if dtype == np.uint8 else 4096
    tf = v.TransferFunction.bake(_keys(rng), width)
    comp = MODES[int(rng.integers(0, len(MODES)))]
    shaded = comp in (v.DVR, v.ISO) and rng.uniform() < 0.4
    p = v.default_params(40, 30)
    p.compositing = comp
    p.shading = v.SHADE_PHONG if shaded else v.SHADE_NONE
    p.sampling_rate = float(rng.uniform(0.5, 4.0))
    p.iso_value = float(rng.uniform(0.05, 0.9))
    p.mida_gamma = float(rng.uniform(-1.0, 1.0))
    brick = [8, 16, 32][int(rng.integers(0, 3))]
    p.empty_space_skipping = int(rng.uniform() < 0.8)
    p.skip_cell_size = [0, 2, 4, 8, 16, brick][int(rng.integers(0, 6))]
    spacing = tuple(float(s) for s in rng.uniform(0.5, 2.0, 3))
    ext = np.array(dims, np.float64) * np.array(spacing)
    centre = ext / 2 - 0.5 * np.array(spacing)
    diag = float(np.linalg.norm(ext)) + 1e-3
    az, el = rng.uniform(0, 2 * np.pi), rng.uniform(-1.2, 1.2)
    eye = centre + rng.uniform(1.0, 2.5) * diag * np.array([np.cos(el) * np.cos(az), np.sin(el),
                                                             np.cos(el) * np.sin(az)])
    p.camera = v.make_camera(tuple(eye), tuple(centre), fovy=float(rng.uniform(20, 60)), near=0.01,
                             far=10 * diag + 10)
    p.light_position[:] = [*eye, 1.0]
    c = Case(ctx, vox, tf, domain, p, spacing, rwm=rwm, brick=brick)
    img, st = c.gpu()
    o32, s32, fh32 = c.oracle(32)
    assert st.samples == s32.sum()
    if shaded:
        assert np.abs(img - o32).max() <= 1e-4
    else:
        np.testing.assert_array_equal(_bits(img), _bits(o32))
    if comp in (v.DVR, v.MIP, v.ISO):
        o64, s64, fh64 = c.oracle(64)
        assert_fp64_parity(img, o32, s32, fh32, o64, s64, fh64, comp, c.step, shaded=shaded, sigs=c.sigs)
