"""The empty-space distance field (volume.cu: occ_dist_x_kernel,
occ_dist_axis_kernel): per skip cell the Chebyshev distance, in cells, to the
nearest occupied cell, capped at 16. The march jumps the box of radius d - 1
around an empty cell at distance d, so a distance above the true one would
skip occupied cells.

The kernels compute it in three separable passes -- along x the distance to
the row's nearest occupied cell, then along y and along z the minimum over
offsets k (|k| < 16) of max(|k|, previous pass at c + k). The CPU tests
restate those passes in numpy and hold them to a brute-force minimum over
all occupied cells; the GPU test holds the kernels' own output
(vrc_occupancy_distance) to the same brute force."""
import ctypes as C

import numpy as np
import pytest

import voreen_gb300 as v

CAP = 16


def brute_force(occ: np.ndarray) -> np.ndarray:
    """occ: (nz, ny, nx) bool. Chebyshev distance to the nearest True cell, capped."""
    nz, ny, nx = occ.shape
    out = np.full(occ.shape, CAP, np.int64)
    pts = np.argwhere(occ)
    if len(pts) == 0:
        return out
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    for pz, py, px in pts:
        d = np.maximum(np.maximum(np.abs(z - pz), np.abs(y - py)), np.abs(x - px))
        np.minimum(out, d, out=out)
    return np.minimum(out, CAP)


def separable(occ: np.ndarray) -> np.ndarray:
    """The kernels' three passes, in the kernels' order and windows."""
    nz, ny, nx = occ.shape
    d = np.full(occ.shape, CAP, np.int64)
    for k in range(CAP - 1, -1, -1):  # along x: nearest occupied cell of the row
        for s in (-k, k):
            src = np.zeros_like(occ)
            if s >= 0:
                src[:, :, : nx - s] = occ[:, :, s:] if s < nx else False
            else:
                src[:, :, -s:] = occ[:, :, : nx + s] if -s < nx else False
            d[src] = np.minimum(d[src], k)
    for axis in (1, 2):  # along y, then z: min over k of max(|k|, previous)
        prev = d.copy()
        n = occ.shape[2 - axis] if axis == 1 else occ.shape[0]
        ax = 1 if axis == 1 else 0
        for k in range(1, CAP):
            for s in (-k, k):
                if abs(s) >= n:
                    continue
                shifted = np.full(occ.shape, CAP, np.int64)
                sl_dst = [slice(None)] * 3
                sl_src = [slice(None)] * 3
                if s > 0:
                    sl_dst[ax], sl_src[ax] = slice(0, n - s), slice(s, n)
                else:
                    sl_dst[ax], sl_src[ax] = slice(-s, n), slice(0, n + s)
                shifted[tuple(sl_dst)] = prev[tuple(sl_src)]
                d = np.minimum(d, np.maximum(k, shifted))
    return d


@pytest.mark.parametrize("shape,density,seed", [((11, 17, 23), 0.01, 1), ((5, 40, 3), 0.002, 2), ((30, 1, 37), 0.05, 3),
                                                ((9, 9, 9), 0.0, 4), ((24, 20, 36), 0.0015, 5), ((1, 1, 50), 0.04, 6)])
def test_separable_passes_equal_brute_force(shape, density, seed):
    rng = np.random.default_rng(seed)
    occ = rng.random(shape) < density
    np.testing.assert_array_equal(separable(occ), brute_force(occ))


def test_cap_bounds_the_box():
    occ = np.zeros((40, 40, 40), bool)
    occ[0, 0, 0] = True
    d = separable(occ)
    assert d[0, 0, 0] == 0 and d[39, 39, 39] == CAP and d[5, 3, 1] == 5
    np.testing.assert_array_equal(d, brute_force(occ))


@pytest.mark.gpu
@pytest.mark.parametrize("shape,density,seed", [((11, 17, 23), 0.01, 11), ((40, 33, 70), 0.003, 12),
                                                ((64, 64, 64), 0.0005, 13), ((3, 90, 5), 0.02, 14)])
def test_kernel_distance_equals_brute_force(ctx, shape, density, seed):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    occ = rng.random(shape) < density
    flat = occ.reshape(-1)
    words = np.zeros((flat.size + 31) // 32, np.uint32)
    idx = np.flatnonzero(flat)
    np.bitwise_or.at(words, idx >> 5, (np.uint32(1) << (idx & 31).astype(np.uint32)))
    d_bits = torch.from_numpy(words.view(np.int32)).cuda()
    d_out = torch.zeros(flat.size, dtype=torch.uint8, device="cuda")
    nz, ny, nx = shape
    st = v.lib().vrc_occupancy_distance(ctx.handle, C.c_void_p(d_bits.data_ptr()), nx, ny, nz,
                                        C.c_void_p(d_out.data_ptr()))
    assert st == 0
    got = d_out.cpu().numpy().reshape(shape).astype(np.int64)
    np.testing.assert_array_equal(got, brute_force(occ))
