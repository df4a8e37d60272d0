"""Host-resident brick pools on the GPU: view-driven cache refinement and the
half-resolution level of detail.

Without a level of detail every image is bit-equal to the device-resident
render whatever the cache holds; the refinement only decides which bricks
are read from HBM. With the level of detail, bricks without a slot are
sampled from the half-resolution level: all-LOD frames are checked bit for
bit against the FP32 oracle on the oracle's own half-sampled volume, and a
still view must converge to the full-resolution image."""
import numpy as np
import pytest

import oracle
import voreen_gb300 as v
from voreen_gb300 import synth

from helpers import oracle_params

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _setup(ctx, size=(96, 80, 64), image=(160, 120), dist_factor=1.25):
    """16^3 bricks (120 of them) so that a view's working set is a fraction of the pool."""
    w = synth.config2(size=size, image=image, dist_factor=dist_factor)
    host = v.Volume(ctx, w.voxels, w.spacing, placement=v.PLACE_HOST, brick_size=16)
    dev = v.Volume(ctx, w.voxels, w.spacing, brick_size=16)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    nb = int(np.prod(host.brick_minmax()[2]))
    return w, host, dev, tf, host.host_bytes // nb


def test_lod_frame_equals_oracle_on_half_volume(ctx):
    """No cache, level of detail on, no empty-space skipping: every sample
    comes from the half-resolution level, which must equal a render of the
    oracle's half-sampled volume at twice the sampling rate (the same step
    in texture space)."""
    w, host, _, tf, _ = _setup(ctx, size=(96, 80, 64), image=(150, 110))
    host.set_cache_limit(0)
    host.set_lod(True)
    p = w.params(shading=v.SHADE_NONE, empty_space_skipping=0)
    e, x = v.entry_exit(ctx, host, p)
    img, st = v.render(ctx, host, tf, p, e, x, v.OUT_RGBA32F)
    half = oracle.half_sample_mean(w.voxels)
    assert half.shape == (32, 40, 48)
    ov = oracle.make_volume(half, w.spacing)
    op = oracle_params(p)
    op.sampling_rate = 2 * p.sampling_rate
    o32, s32, _ = oracle.render(ov, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain, op, e, x, 32)
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert st.samples == s32.sum()
    # the full-resolution image differs (the level really is coarser)
    full, _ = v.render(ctx, v.Volume(ctx, w.voxels, w.spacing), tf, p, e, x, v.OUT_RGBA32F)
    assert np.abs(full - img).max() > 1e-3


def test_half_level_of_odd_dims(ctx):
    """Odd dimensions (the last block of an axis repeats the edge voxel) and
    8^3 bricks; MIP. The largest dimension is even so the step in texture
    space is the same at twice the rate."""
    w = synth.config2(size=(38, 21, 29), image=(90, 70))
    host = v.Volume(ctx, w.voxels, w.spacing, placement=v.PLACE_HOST, brick_size=8)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    host.set_cache_limit(0)
    host.set_lod(True)
    p = w.params(shading=v.SHADE_NONE, empty_space_skipping=0, compositing=v.MIP)
    e, x = v.entry_exit(ctx, host, p)
    img, st = v.render(ctx, host, tf, p, e, x, v.OUT_RGBA32F)
    half = oracle.half_sample_mean(w.voxels)
    assert half.shape == (15, 11, 19)
    ov = oracle.make_volume(half, w.spacing)
    op = oracle_params(p)
    op.sampling_rate = 2 * p.sampling_rate
    o32, s32, _ = oracle.render(ov, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain, op, e, x, 32)
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert st.samples == s32.sum()


def test_refinement_without_lod_is_exact_and_converges(ctx):
    """A cache smaller than the TF-reachable set: images stay bit-equal to
    the device-resident render every frame; a budget one brick above the
    view's working set drives misses to zero after one refinement."""
    w, host, dev, tf, brick_bytes = _setup(ctx, dist_factor=0.75)
    p = w.params(shading=v.SHADE_PHONG, entry_exit_mode=v.EE_ANALYTIC)
    ref, sref = v.render(ctx, dev, tf, p, None, None, v.OUT_RGBA32F)
    host.set_cache_limit(brick_bytes)  # one slot: misses = the working set (minus at most one brick)
    img, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
    np.testing.assert_array_equal(_bits(img), _bits(ref))
    cached, reach, missed = host.cache_info()
    assert cached == 1 and reach > 4
    work = missed + 1
    assert 1 < work <= reach
    host.set_cache_limit(brick_bytes * (work + 2))
    misses = []
    for _ in range(4):
        img, st = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
        np.testing.assert_array_equal(_bits(img), _bits(ref))
        assert st.samples == sref.samples
        misses.append(host.cache_info()[2])
    assert misses[-1] == 0 and misses[-2] == 0, misses
    assert misses == sorted(misses, reverse=True), misses


def test_lod_with_full_cache_is_exact(ctx):
    """Every brick the TF can reach cached: no sample needs the level of
    detail, so the image is the full-resolution one."""
    w, host, dev, tf, _ = _setup(ctx)
    host.set_lod(True)
    for shading in (v.SHADE_NONE, v.SHADE_PHONG):
        p = w.params(shading=shading, entry_exit_mode=v.EE_ANALYTIC)
        ref, _ = v.render(ctx, dev, tf, p, None, None, v.OUT_RGBA32F)
        img, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
        np.testing.assert_array_equal(_bits(img), _bits(ref))
        cached, reach, missed = host.cache_info()
        assert cached == reach and missed == 0


def test_lod_refinement_converges_to_full_resolution(ctx):
    """A partial cache with the level of detail: the first frames mix
    resolutions, and once a frame reads no brick without a slot it is the
    full-resolution image."""
    w, host, dev, tf, brick_bytes = _setup(ctx, dist_factor=0.75)
    p = w.params(shading=v.SHADE_PHONG, entry_exit_mode=v.EE_ANALYTIC)
    ref, _ = v.render(ctx, dev, tf, p, None, None, v.OUT_RGBA32F)
    host.set_cache_limit(brick_bytes)
    v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
    work = host.cache_info()[2] + 1
    reach = host.cache_info()[1]
    budget = min(reach - 1, work + 4)
    assert work < budget, (work, reach)  # the view sees part of the reachable bricks
    host.set_cache_limit(brick_bytes * budget)
    host.set_lod(True)
    done = False
    for _ in range(8):
        img, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
        if host.cache_info()[2] == 0:
            np.testing.assert_array_equal(_bits(img), _bits(ref))
            done = True
            break
    assert done


def test_lod_rejected_for_device_pool(ctx):
    w = synth.config1(size=(24, 24, 24))
    vol = v.Volume(ctx, w.voxels, w.spacing)
    with pytest.raises(v.VrcError):
        vol.set_lod(True)


def test_upload_budget_streams_bricks_in(ctx):
    """A per-render upload budget of 3 bricks: the cache grows by at most 3
    bricks a render, every image stays exact, and the cache ends up holding
    every brick the TF reaches."""
    w, host, dev, tf, brick_bytes = _setup(ctx)
    host.set_cache_upload_budget(3 * brick_bytes)
    p = w.params(shading=v.SHADE_PHONG, entry_exit_mode=v.EE_ANALYTIC)
    ref, _ = v.render(ctx, dev, tf, p, None, None, v.OUT_RGBA32F)
    prev = 0
    for i in range(200):
        img, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
        np.testing.assert_array_equal(_bits(img), _bits(ref))
        cached, reach, missed = host.cache_info()
        assert cached - prev <= 3
        prev = cached
        if cached == reach:
            break
    assert cached == reach and i >= (reach - 1) // 3


def test_upload_budget_with_lod_converges(ctx):
    w, host, dev, tf, brick_bytes = _setup(ctx)
    host.set_cache_upload_budget(4 * brick_bytes)
    host.set_lod(True)
    p = w.params(shading=v.SHADE_NONE, entry_exit_mode=v.EE_ANALYTIC)
    ref, _ = v.render(ctx, dev, tf, p, None, None, v.OUT_RGBA32F)
    first, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
    for _ in range(200):
        img, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
        cached, reach, missed = host.cache_info()
        if cached == reach and missed == 0:
            break
    # the last render read only cached bricks (misses are counted after it)
    img, _ = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
    np.testing.assert_array_equal(_bits(img), _bits(ref))
    assert not np.array_equal(_bits(first), _bits(ref))


@pytest.mark.parametrize("seed", range(8))
def test_random_cache_settings_are_exact(ctx, seed):
    """Random cache budgets, upload budgets, brick sizes, modes and TF changes
    on a host-resident pool: every frame equals the device-resident one."""
    rng = np.random.default_rng(900 + seed)
    brick = [16, 32][seed % 2]
    w = synth.config2(size=(72, 64, 56), image=(96, 72), dist_factor=float(rng.uniform(0.7, 1.4)),
                      azimuth=float(rng.uniform(0, 360)))
    host = v.Volume(ctx, w.voxels, w.spacing, placement=v.PLACE_HOST, brick_size=brick)
    dev = v.Volume(ctx, w.voxels, w.spacing, brick_size=brick)
    nb = int(np.prod(host.brick_minmax()[2]))
    bb = host.host_bytes // nb
    host.set_cache_limit(int(bb * rng.integers(1, nb + 1)))
    host.set_cache_upload_budget(int(bb * rng.integers(1, 8)) if rng.uniform() < 0.7 else 0)
    keys2 = [(0.0, (0, 0, 0, 0)), (float(rng.uniform(0.2, 0.6)), (0, 0, 0, 0)), (0.8, (250, 200, 90, 160)),
             (1.0, (255, 255, 255, 255))]
    tfs = [v.TransferFunction(ctx, v.TransferFunction.bake(k, w.tf_width), w.domain) for k in (w.tf_keys, keys2)]
    comp = [v.DVR, v.MIP, v.ISO][int(rng.integers(0, 3))]
    p = w.params(entry_exit_mode=v.EE_ANALYTIC, compositing=comp,
                 shading=v.SHADE_PHONG if comp == v.DVR else v.SHADE_NONE)
    for frame in range(5):
        tf = tfs[int(rng.integers(0, 2))]
        a, sa = v.render(ctx, host, tf, p, None, None, v.OUT_RGBA32F)
        b, sb = v.render(ctx, dev, tf, p, None, None, v.OUT_RGBA32F)
        np.testing.assert_array_equal(_bits(a), _bits(b))
        assert sa.samples == sb.samples


@pytest.mark.parametrize("level,dims,brick", [(2, (96, 80, 64), 16), (3, (96, 72, 40), 8), (2, (76, 42, 58), 8)])
def test_deeper_lod_level_equals_oracle_pyramid(ctx, level, dims, brick):
    """Level k of the pyramid: with no cache every sample comes from the
    2^-k level, which must equal the oracle's render of the volume
    half-sampled k times (HalfSampleMean applied level by level, each with
    its own edge clamping) at 2^k times the sampling rate -- the same step in
    texture space (the largest dimension is a multiple of 2^k). Switching
    the level rebuilds it; level 1 afterwards is the half-resolution level
    again."""
    w = synth.config2(size=dims, image=(120, 96))
    host = v.Volume(ctx, w.voxels, w.spacing, placement=v.PLACE_HOST, brick_size=brick)
    tf_rgba = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    tf = v.TransferFunction(ctx, tf_rgba, w.domain)
    host.set_cache_limit(0)
    p = w.params(shading=v.SHADE_NONE, empty_space_skipping=0)
    e, x = v.entry_exit(ctx, host, p)
    for k in (level, 1):
        host.set_lod(k)
        img, st = v.render(ctx, host, tf, p, e, x, v.OUT_RGBA32F)
        vox = w.voxels
        for _ in range(k):
            vox = oracle.half_sample_mean(vox)
        ov = oracle.make_volume(np.ascontiguousarray(vox), w.spacing)
        op = oracle_params(p)
        op.sampling_rate = (2 ** k) * p.sampling_rate
        o32, s32, _ = oracle.render(ov, tf_rgba, w.domain, op, e, x, 32)
        np.testing.assert_array_equal(_bits(img), _bits(o32), err_msg=f"level {k}")
        assert st.samples == s32.sum()
        assert (img[..., 3] > 0).mean() > 0.02
    host.set_lod(0)
    with pytest.raises(v.VrcError):
        host.set_lod(7)
    host.close()
