"""GPU parity: the CUDA march through the C ABI against the CPU oracle on the
same seeded inputs. Unshaded paths must match the FP32 oracle bit for bit;
every path must be within 1/255 per channel of the FP64 oracle on rays where
FP32 and FP64 take the same discrete decisions."""
import numpy as np
import pytest

import oracle
import voreen_gb300 as v
from voreen_gb300 import synth

from helpers import Case, TOL, assert_fp64_parity, oracle_entry_exit

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _c1_case(ctx, **kw):
    w = synth.config1(**kw)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    return w, Case(ctx, w.voxels, tf, w.domain, w.params(), w.spacing)


def test_config1_full_size_bit_exact(ctx):
    """Plain DVR, 128^3 u8, 512x512 (the CPU-runnable configuration)."""
    w, c = _c1_case(ctx)
    img, st = c.gpu()
    o32, s32, fh32 = c.oracle(32)
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert st.samples == s32.sum()
    o64, s64, fh64 = c.oracle(64)
    assert_fp64_parity(img, o32, s32, fh32, o64, s64, fh64, v.DVR, c.step, label="C1 128^3 u8 512x512 DVR", sigs=c.sigs)


@pytest.mark.parametrize("comp", [v.DVR, v.MIP, v.ISO])
def test_ct_shells_unshaded_bit_exact(ctx, comp):
    w = synth.config2(size=(96, 80, 72), image=(200, 150), compositing=comp)
    p = w.params(shading=v.SHADE_NONE, iso_value=0.3)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, p, w.spacing)
    img, st = c.gpu()
    o32, s32, fh32 = c.oracle(32)
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert st.samples == s32.sum()
    o64, s64, fh64 = c.oracle(64)
    assert_fp64_parity(img, o32, s32, fh32, o64, s64, fh64, comp, c.step, label=f"shells 96x80x72 mode {comp}", sigs=c.sigs)


@pytest.mark.parametrize("comp", [v.DVR, v.ISO])
def test_ct_shells_phong(ctx, comp):
    """Phong + central differences: the gradient is computed from the brick
    stencil (index shifts) instead of six texture-space lookups, so results
    are close to, not bit-equal with, the FP32 oracle."""
    w = synth.config2(size=(96, 96, 80), image=(220, 160), compositing=comp)
    p = w.params(shading=v.SHADE_PHONG, iso_value=0.3)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, p, w.spacing)
    img, st = c.gpu()
    o32, s32, fh32 = c.oracle(32)
    assert st.samples == s32.sum()
    assert st.samples_shaded > 0
    assert np.abs(img - o32).max() <= 1e-4
    o64, s64, fh64 = c.oracle(64)
    assert_fp64_parity(img, o32, s32, fh32, o64, s64, fh64, comp, c.step, shaded=True,
                       label=f"shells 96x96x80 Phong mode {comp}", sigs=c.sigs)


def test_float_volume_and_rwm(ctx):
    """float32 blobs with a non-identity real-world mapping and a domain."""
    vox = v.synth_volume(0, v.F32, (40, 33, 27), 77)
    keys = [(0.0, (0, 50, 200, 0)), (0.3, (20, 200, 40, 0)), (0.6, (220, 200, 10, 90)), (1.0, (255, 0, 0, 200))]
    tf = v.TransferFunction.bake(keys, 4096)
    p = v.default_params(96, 80)
    p.camera = v.make_camera((60, 40, 90), (20, 16, 13))
    rwm = (2.0, -0.25)
    c = Case(ctx, vox, tf, (-0.2, 1.5), p, spacing=(1.2, 0.9, 1.1), rwm=rwm)
    img, st = c.gpu()
    o32, s32, fh32 = c.oracle(32)
    np.testing.assert_array_equal(_bits(img), _bits(o32))


@pytest.mark.parametrize("dims,brick", [((1, 1, 1), 8), ((2, 3, 5), 8), ((40, 40, 1), 16), ((17, 9, 33), 8),
                                        ((65, 31, 7), 64), ((70, 70, 70), 32)])
def test_odd_shapes_and_brick_sizes(ctx, dims, brick):
    X, Y, Z = dims
    rng = np.random.default_rng(X * 100 + Y * 10 + Z)
    vox = rng.integers(0, 256, size=(Z, Y, X), dtype=np.uint8)
    keys = [(0.0, (0, 0, 255, 0)), (0.2, (0, 255, 0, 40)), (1.0, (255, 0, 0, 200))]
    tf = v.TransferFunction.bake(keys, 256)
    p = v.default_params(64, 48)
    diag = float(np.sqrt(X * X + Y * Y + Z * Z))
    p.camera = v.make_camera((X * 0.5 + diag, Y * 0.5 + 0.6 * diag, Z * 0.5 + 1.2 * diag), (X / 2, Y / 2, Z / 2),
                             near=0.1, far=10 * diag + 10)
    p.sampling_rate = 3.0
    c = Case(ctx, vox, tf, (0.0, 1.0), p, brick=brick)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32)
    assert s32.sum() > 0
    np.testing.assert_array_equal(_bits(img), _bits(o32))


def test_default_skip_cell_is_the_finest_level(ctx):
    """skip_cell_size 0 takes the 2^3 cells where the volume holds them: the
    same fetched samples and pixels as an explicit 2, fewer fetches than 4^3
    cells, and every frame equal to the render without skipping."""
    w = synth.config2(size=(96, 88, 80), image=(200, 150))
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, w.params(), w.spacing)
    a, sa = c.gpu(skip_cell_size=0)
    b, sb = c.gpu(skip_cell_size=2)
    d, sd = c.gpu(skip_cell_size=4)
    e, se = c.gpu(empty_space_skipping=0, skip_cell_size=0)
    for img in (b, d, e):
        np.testing.assert_array_equal(_bits(a), _bits(img))
    assert sa.samples_fetched == sb.samples_fetched < sd.samples_fetched < se.samples_fetched
    assert sa.samples == sb.samples == sd.samples == se.samples


@pytest.mark.parametrize("cell,compositing", [(2, v.DVR), (4, v.DVR), (8, v.DVR), (32, v.DVR), (4, v.MIP), (2, v.ISO)])
def test_sparse_volume_skipping_is_exact(ctx, cell, compositing):
    """Sparse tubes (most skip cells empty, occupied ones in thin strands):
    jumping the empty box around a cell that the distance to the nearest
    occupied cell guarantees leaves every pixel and the sample count
    unchanged, and (cells of 8^3 or less) fetches less than half the
    samples."""
    vox = v.synth_tubes_device((192, 160, 128), 12, 77).cpu().numpy()
    lo, hi = float(vox.min()) / 65535.0, float(vox.max()) / 65535.0
    keys, domain = synth.tubes_tf(78, 2, (lo, hi))
    tf = v.TransferFunction.bake(keys, 4096)
    X, Y, Z = 192, 160, 128
    p = v.default_params(256, 192)
    p.sampling_rate, p.shading, p.compositing = 1.5, v.SHADE_PHONG, compositing
    p.entry_exit_mode, p.skip_cell_size = v.EE_ANALYTIC, cell
    pos, focus, near, far = synth.orbit_camera((X, Y, Z), (1.0, 1.0, 1.0), 30.0, 25.0, 1.2)
    p.camera = v.make_camera(pos, focus, near=near, far=far)
    c = Case(ctx, vox, tf, domain, p, (1.0, 1.0, 1.0), brick=32)
    a, sa = c.gpu(empty_space_skipping=1)
    b, sb = c.gpu(empty_space_skipping=0)
    np.testing.assert_array_equal(_bits(a), _bits(b))
    assert sa.samples == sb.samples
    assert (a[..., 3] > 0).mean() > 0.01
    if compositing == v.DVR and cell <= 8:
        assert sa.samples_fetched < 0.5 * sb.samples_fetched


@pytest.mark.parametrize("cell,brick,shading", [(8, 32, v.SHADE_NONE), (16, 32, v.SHADE_PHONG), (32, 32, v.SHADE_NONE),
                                                (8, 16, v.SHADE_PHONG), (64, 64, v.SHADE_NONE),
                                                (4, 32, v.SHADE_PHONG), (4, 16, v.SHADE_NONE),
                                                (2, 32, v.SHADE_PHONG), (2, 16, v.SHADE_NONE)])
def test_empty_space_skipping_is_exact(ctx, cell, brick, shading):
    """Skipping empty cells (2^3, 4^3, 8^3, 16^3 or whole bricks) leaves every
    pixel and the sample count unchanged."""
    w = synth.config2(size=(130, 128, 127), image=(256, 192))
    p = w.params(shading=shading, skip_cell_size=cell)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, p, w.spacing, brick=brick)
    a, sa = c.gpu(empty_space_skipping=1)
    b, sb = c.gpu(empty_space_skipping=0)
    np.testing.assert_array_equal(_bits(a), _bits(b))
    assert sa.samples == sb.samples
    assert sa.samples_fetched <= sb.samples_fetched
    if cell <= 16:
        assert sa.samples_fetched < 0.9 * sb.samples_fetched


def test_brick_minmax_and_volume_minmax(ctx):
    vox = v.synth_volume(1, v.U16, (70, 45, 33), 5)
    vol = v.Volume(ctx, vox, brick_size=16)
    mn, mx, nb = vol.brick_minmax()
    ov = oracle.make_volume(vox)
    omn, omx, onb = oracle.brick_minmax(ov, 16, 1)
    assert tuple(nb) == tuple(onb)
    np.testing.assert_array_equal(mn, omn)
    np.testing.assert_array_equal(mx, omx)
    lo, hi = vol.minmax()
    assert lo == np.float32(vox.min()) / np.float32(65535) and hi == np.float32(vox.max()) / np.float32(65535)


def test_analytic_entry_exit_matches_buffers(ctx):
    """In-kernel analytic entry/exit equals rendering from the entry/exit
    images the library writes; those agree with the FP64 oracle's rays."""
    w = synth.config2(size=(64, 64, 64), image=(160, 120), compositing=v.DVR)
    p = w.params(shading=v.SHADE_PHONG)
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, p, w.spacing)
    e, x = v.entry_exit(ctx, c.vol, p)
    oe, ox = oracle_entry_exit(c.vol.desc, p)
    hit = (e[..., 3] > 0) & (oe[..., 3] > 0)
    assert ((e[..., 3] > 0) != (oe[..., 3] > 0)).sum() <= 0.002 * hit.sum() + 2
    assert np.abs(e[hit] - oe[hit]).max() < 2e-5 and np.abs(x[hit] - ox[hit]).max() < 2e-5
    pa = w.params(shading=v.SHADE_PHONG, entry_exit_mode=v.EE_ANALYTIC)
    img_a, _ = v.render(ctx, c.vol, c.tf, pa, None, None, v.OUT_RGBA32F)
    img_b, _ = v.render(ctx, c.vol, c.tf, p, e, x, v.OUT_RGBA32F)
    np.testing.assert_array_equal(_bits(img_a), _bits(img_b))


def test_clip_region_entry_exit(ctx):
    """Proxy-geometry clipping (OptimizedProxyGeometry clipRegion): analytic
    entry/exit on the clipped cube against the FP64 oracle's, rendering from
    them equals rendering in analytic mode, and the march only reaches the
    clip box (+ the half-voxel border)."""
    w = synth.config2(size=(64, 60, 56), image=(160, 120), compositing=v.DVR)
    p = w.params(shading=v.SHADE_NONE)
    p.enable_clipping = 1
    p.clip_llf[:] = [8, 5, 20]
    p.clip_urb[:] = [40, 59, 50]
    tf = v.TransferFunction.bake(w.tf_keys, w.tf_width)
    c = Case(ctx, w.voxels, tf, w.domain, p, w.spacing, entry=np.zeros((1,)), exit_pts=np.zeros((1,)))
    e, x = v.entry_exit(ctx, c.vol, p)
    dims = np.array(c.vol.dims, np.float64)
    lo = np.maximum(0.0, np.array([8, 5, 20]) / dims)
    hi = np.minimum(1.0, (np.array([40, 59, 50]) + 1.0) / dims)
    _, _, inv = v.camera_matrices(p.camera, c.vol.desc, p.width, p.height)
    oe, ox = oracle.entry_exit(inv, p.width, p.height, False, box=(lo, hi))
    hit = (e[..., 3] > 0) & (oe[..., 3] > 0)
    assert hit.sum() > 100
    assert ((e[..., 3] > 0) != (oe[..., 3] > 0)).sum() <= 0.002 * hit.sum() + 2
    assert np.abs(e[hit] - oe[hit]).max() < 2e-5 and np.abs(x[hit] - ox[hit]).max() < 2e-5
    pts = np.concatenate([e[hit][:, :3], x[hit][:, :3]])
    assert np.all(pts >= lo - 1e-6) and np.all(pts <= hi + 1e-6)
    img_b, _ = v.render(ctx, c.vol, c.tf, p, e, x, v.OUT_RGBA32F)
    p.entry_exit_mode = v.EE_ANALYTIC
    img_a, _ = v.render(ctx, c.vol, c.tf, p, None, None, v.OUT_RGBA32F)
    np.testing.assert_array_equal(_bits(img_a), _bits(img_b))
    o32, _, _ = c.oracle(32, entry=e, exit_pts=x)
    np.testing.assert_array_equal(_bits(img_b), _bits(o32))
    p.clip_llf[0] = 50  # llf > urb
    with pytest.raises(v.VrcError, match="INVALID_ARG"):
        v.render(ctx, c.vol, c.tf, p, None, None, v.OUT_RGBA32F)


def test_output_formats(ctx):
    w, c = _c1_case(ctx, size=(48, 40, 36), image=(96, 64))
    f32, _ = c.gpu(v.OUT_RGBA32F)
    u8, _ = c.gpu(v.OUT_RGBA8)
    u16, _ = c.gpu(v.OUT_RGBA16)
    q = lambda a, s: np.floor(np.clip(a, 0, 1) * np.float32(s) + np.float32(0.5))
    np.testing.assert_array_equal(u8.astype(np.float32), q(f32, 255))
    np.testing.assert_array_equal(u16.astype(np.float32), q(f32, 65535))


def test_degenerate_and_background_rays(ctx):
    """cpuraycaster.cpp:184 background (entry == exit == 0) and :226-227
    degenerate rays (entry == exit != 0: one sample, tend = step / 2)."""
    rng = np.random.default_rng(3)
    vox = rng.integers(0, 256, size=(20, 20, 20), dtype=np.uint8)
    tf = v.TransferFunction.bake([(0.0, (255, 255, 255, 255)), (1.0, (255, 0, 0, 255))], 256)
    H, W = 8, 16
    e = rng.uniform(0, 1, (H, W, 4)).astype(np.float32)
    x = rng.uniform(0, 1, (H, W, 4)).astype(np.float32)
    e[..., 3] = x[..., 3] = 1
    e[0, :] = 0
    x[0, :] = 0                      # background row
    x[1, :] = e[1, :]                # degenerate rays
    e[2, :, :3] = 0                  # entry at the origin, exit elsewhere
    x[3, :, :3] = 0                  # exit at the origin
    p = v.default_params(W, H)
    c = Case(ctx, vox, tf, (0.0, 1.0), p, entry=e, exit_pts=x)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32)
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert (s32[0] == 0).all() and (s32[1] == 1).all() and (img[0] == 0).all()


def test_errors_are_statuses(ctx):
    vox = np.zeros((4, 4, 4), np.uint8)
    vol = v.Volume(ctx, vox)
    tf = v.TransferFunction(ctx, np.zeros((256, 4), np.uint8))
    p = v.default_params(8, 8)
    with pytest.raises(v.VrcError) as ei:
        v.render(ctx, vol, tf, p, None, None)       # buffer mode without entry/exit
    assert ei.value.status == 6
    p.sampling_rate = 0.0
    e = np.zeros((8, 8, 4), np.float32)
    with pytest.raises(v.VrcError) as ei:
        v.render(ctx, vol, tf, p, e, e)
    assert ei.value.status == 1
    with pytest.raises(v.VrcError):
        v.Volume(ctx, vox, brick_size=12)
    with pytest.raises(v.VrcError):
        v.TransferFunction(ctx, np.zeros((5000, 4), np.uint8))


def test_device_tube_volume_parity(ctx):
    """The large-volume family (sparse tubes generated on the device) at a
    reduced size: unshaded bit-exact, Phong within 1e-4, most cells empty."""
    torch = pytest.importorskip("torch")
    dims = (192, 160, 128)
    vox = v.synth_tubes_device(dims, 8, 77)
    assert vox.dtype == torch.uint16
    host = vox.cpu().numpy()
    assert host.max() <= 4095
    assert (host > 1000).mean() < 0.5
    lo, hi = float(host.min()) / 65535, float(host.max()) / 65535
    keys, domain = synth.tubes_tf(5, 2, (lo, hi))
    tf = v.TransferFunction.bake(keys, 4096)
    pos, focus, near, far = synth.orbit_camera(dims, (1, 1, 1), 40.0, 20.0, 1.3)
    p = v.default_params(160, 120)
    p.sampling_rate = 1.5
    p.camera = v.make_camera(pos, focus, near=near, far=far)
    p.light_position[:] = [*pos, 1.0]
    c = Case(ctx, host, tf, domain, p)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32)
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert st.samples_fetched < 0.5 * st.samples
    img, st = c.gpu(shading=v.SHADE_PHONG)
    o32, s32, _ = c.oracle(32)
    assert np.abs(img - o32).max() <= 1e-4


@pytest.mark.parametrize("from_device", [False, True])
def test_host_placed_brick_pool(ctx, from_device):
    """A brick pool in pinned host memory (read by the march through its mapped
    address) renders exactly as the device-resident one, and no device copy of
    the voxels is kept."""
    torch = pytest.importorskip("torch")
    w = synth.config2(size=(97, 80, 66), image=(160, 120))
    src = torch.from_numpy(w.voxels).cuda() if from_device else w.voxels
    a = v.Volume(ctx, src, w.spacing, placement=v.PLACE_HOST)
    b = v.Volume(ctx, w.voxels, w.spacing)
    assert a.minmax() == b.minmax()
    assert a.host_bytes > 0 and a.device_bytes < b.device_bytes and b.host_bytes == 0
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    for shading in (v.SHADE_NONE, v.SHADE_PHONG):
        p = w.params(entry_exit_mode=v.EE_ANALYTIC, shading=shading)
        ia, sa = v.render(ctx, a, tf, p, None, None, v.OUT_RGBA32F)
        ib, sb = v.render(ctx, b, tf, p, None, None, v.OUT_RGBA32F)
        np.testing.assert_array_equal(_bits(ia), _bits(ib))
        assert sa.samples == sb.samples


@pytest.mark.gpu
def test_host_pool_device_cache(ctx):
    """The device brick cache of a host-placed pool never changes an image:
    with no cache, a partial one (the rest read from the host pool) and a
    full one, across TF changes that keep part of the cached set, and for
    DVR (with and without shading) and MIP."""
    pytest.importorskip("torch")
    w = synth.config2(size=(97, 80, 66), image=(160, 120))
    a = v.Volume(ctx, w.voxels, w.spacing, placement=v.PLACE_HOST)
    b = v.Volume(ctx, w.voxels, w.spacing)
    nb = int(np.prod(a.brick_minmax()[2]))
    brick_bytes = a.host_bytes // nb
    keys2 = [(0.0, (0, 0, 0, 0)), (0.55, (0, 0, 0, 0)), (0.7, (250, 200, 90, 160)), (1.0, (255, 255, 255, 255))]
    tfs = [v.TransferFunction(ctx, v.TransferFunction.bake(k, w.tf_width), w.domain) for k in (w.tf_keys, keys2)]
    cases = [(v.DVR, v.SHADE_NONE), (v.DVR, v.SHADE_PHONG), (v.MIP, v.SHADE_NONE)]
    seen = set()
    for limit in (None, 0, "half", None):
        if limit == "half":
            a.set_cache_limit(brick_bytes * max(1, a.cache_info()[1] // 2))
        elif limit is not None:
            a.set_cache_limit(limit)
        else:
            a.set_cache_limit(2**62)
        for tf in tfs:
            for comp, shading in cases:
                p = w.params(entry_exit_mode=v.EE_ANALYTIC, shading=shading, compositing=comp)
                ia, sa = v.render(ctx, a, tf, p, None, None, v.OUT_RGBA32F)
                ib, sb = v.render(ctx, b, tf, p, None, None, v.OUT_RGBA32F)
                np.testing.assert_array_equal(_bits(ia), _bits(ib))
                assert sa.samples == sb.samples
                cached, reach, _ = a.cache_info()
                assert 0 < reach <= nb and cached <= reach
                if limit == 0:
                    assert cached == 0
                elif limit == "half":
                    assert 0 < cached < reach
                else:
                    assert cached == reach
                seen.add((limit, cached == reach))
    assert len(seen) == 3


@pytest.mark.gpu
def test_pinned_host_buffers_in_place(ctx):
    """Pinned host entry/exit points and output are used in place by the
    kernel (mapped addresses); pageable ones are staged. Every combination
    gives the same image."""
    torch = pytest.importorskip("torch")
    w = synth.config2(size=(90, 77, 64), image=(150, 110))
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    p = w.params(shading=v.SHADE_PHONG)
    e, x = v.entry_exit(ctx, vol, p)

    def pin(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    for fmt, dt in ((v.OUT_RGBA8, np.uint8), (v.OUT_RGBA32F, np.float32)):
        ref, sr = v.render(ctx, vol, tf, p, e, x, fmt)
        for ee in ((pin(e), pin(x)), (pin(e), x), (e, pin(x))):
            for o in (None, pin(np.zeros(ref.shape, dt))):
                img, st = v.render(ctx, vol, tf, p, ee[0], ee[1], fmt, o)
                np.testing.assert_array_equal(img, ref)
                assert st.samples == sr.samples


@pytest.mark.gpu
def test_occupancy_reused_across_frames(ctx):
    """The empty-space occupancy bits and their distance field are computed
    once per (volume, TF, cell edge) and reused by later frames (a frame
    that builds them launches the occupancy kernel, three distance passes
    and the march); switching TFs, volumes or cell edges recomputes them,
    and every image equals a fresh context's."""
    w = synth.config2(size=(80, 72, 64), image=(120, 90))
    keys2 = [(0.0, (0, 0, 0, 0)), (0.5, (0, 0, 0, 0)), (0.7, (250, 200, 90, 160)), (1.0, (255, 255, 255, 255))]
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tfa = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    tfb = v.TransferFunction(ctx, v.TransferFunction.bake(keys2, w.tf_width), w.domain)
    p = w.params(entry_exit_mode=v.EE_ANALYTIC, shading=v.SHADE_PHONG)

    def fresh(keys, cell=0):
        c2 = v.Context(0)
        vol2 = v.Volume(c2, w.voxels, w.spacing)
        tf2 = v.TransferFunction(c2, v.TransferFunction.bake(keys, w.tf_width), w.domain)
        q = w.params(entry_exit_mode=v.EE_ANALYTIC, shading=v.SHADE_PHONG, skip_cell_size=cell)
        img, _ = v.render(c2, vol2, tf2, q, None, None, v.OUT_RGBA32F)
        tf2.close()  # a context's objects go before the context
        vol2.close()
        c2.close()
        return img

    ref_a, ref_b = fresh(w.tf_keys), fresh(keys2)
    img, st = v.render(ctx, vol, tfa, p, None, None, v.OUT_RGBA32F)
    assert st.kernel_launches == 5 and np.array_equal(_bits(img), _bits(ref_a))
    img, st = v.render(ctx, vol, tfa, p, None, None, v.OUT_RGBA32F)
    assert st.kernel_launches == 1 and np.array_equal(_bits(img), _bits(ref_a))
    img, st = v.render(ctx, vol, tfb, p, None, None, v.OUT_RGBA32F)
    assert st.kernel_launches == 5 and np.array_equal(_bits(img), _bits(ref_b))
    img, st = v.render(ctx, vol, tfa, p, None, None, v.OUT_RGBA32F)
    assert st.kernel_launches == 5 and np.array_equal(_bits(img), _bits(ref_a))
    p.skip_cell_size = 16
    img, st = v.render(ctx, vol, tfa, p, None, None, v.OUT_RGBA32F)
    assert st.kernel_launches == 5 and np.array_equal(_bits(img), _bits(fresh(w.tf_keys, 16)))
    # a TF destroyed and re-created (possibly at the same address) is a new TF
    tfa.close()
    tfc = v.TransferFunction(ctx, v.TransferFunction.bake(keys2, w.tf_width), w.domain)
    img, st = v.render(ctx, vol, tfc, p, None, None, v.OUT_RGBA32F)
    assert st.kernel_launches == 5


@pytest.mark.parametrize("skipping", [1, 0])
def test_loop_cap(ctx, skipping):
    """cpuraycaster.cpp:239: a ray stops after 255 * 255 loop iterations. At
    rate 3000 on a 32^3 volume (step 1/96000) the rays need ~1e5 samples;
    the cap, also inside closed-form jumps over empty cells, matches the
    oracle bit for bit."""
    rng = np.random.default_rng(11)
    vox = rng.integers(0, 256, size=(32, 32, 32), dtype=np.uint8)
    vox[:, :, :16] //= 4  # an empty half under the TF below
    tf = v.TransferFunction.bake([(0.0, (0, 0, 0, 0)), (0.3, (0, 0, 0, 0)), (0.31, (200, 90, 40, 1)),
                                  (1.0, (40, 90, 200, 2))], 256)
    p = v.default_params(6, 4)
    p.sampling_rate = 3000.0
    p.empty_space_skipping = skipping
    p.camera = v.make_camera((60.0, 40.0, 70.0), (16.0, 16.0, 16.0), near=1.0, far=300.0, fovy=12.0)
    c = Case(ctx, vox, tf, (0.0, 1.0), p)
    img, st = c.gpu()
    o32, s32, _ = c.oracle(32)
    assert s32.max() == 255 * 255  # some rays reach the cap
    np.testing.assert_array_equal(_bits(img), _bits(o32))
    assert st.samples == s32.sum()


@pytest.mark.parametrize("kind", ["u16_shells", "f32_signed", "u8_plateaus", "f32_negative_scale"])
def test_mip_cell_skipping_is_exact(ctx, kind):
    """MIP skips cells whose largest value cannot raise the ray's maximum: the
    image and the sample count equal the render without skipping and the
    FP32 oracle bit for bit, including negative values, a negative
    real-world offset, plateaus (samples equal to the cell maximum) and a
    negative scale (where that skipping is off)."""
    rng = np.random.default_rng(21)
    rwm = (1.0, 0.0)
    if kind == "u16_shells":
        w = synth.config2(size=(96, 80, 72), image=(160, 120), compositing=v.MIP)
        vox, keys, dom, spacing = w.voxels, w.tf_keys, w.domain, w.spacing
    else:
        spacing = (1.0, 1.0, 1.0)
        if kind == "u8_plateaus":
            vox = (rng.integers(0, 6, size=(40, 48, 56)) * 40).astype(np.uint8)  # few distinct levels
            dom = (0.0, 1.0)
        else:
            vox = rng.normal(0.0, 1.0, size=(40, 48, 56)).astype(np.float32)
            rwm = (2.0, -0.5) if kind == "f32_signed" else (-1.5, 0.25)
            dom = (-3.0, 3.0)
        keys = [(0.0, (0, 0, 255, 0)), (0.4, (0, 255, 0, 30)), (1.0, (255, 0, 0, 200))]
    tf = v.TransferFunction.bake(keys, 256 if vox.dtype == np.uint8 else 4096)
    p = v.default_params(120, 90)
    X, Y, Z = vox.shape[2], vox.shape[1], vox.shape[0]
    d = float(np.sqrt(X * X + Y * Y + Z * Z))
    p.camera = v.make_camera((X * 0.5 + 0.9 * d, Y * 0.5 + 0.5 * d, Z * 0.5 + 1.1 * d), (X / 2, Y / 2, Z / 2),
                             near=0.1, far=10 * d)
    p.compositing = v.MIP
    c = Case(ctx, vox, tf, dom, p, spacing, rwm=rwm)
    a, sa = c.gpu(empty_space_skipping=1)
    b, sb = c.gpu(empty_space_skipping=0)
    np.testing.assert_array_equal(_bits(a), _bits(b))
    assert sa.samples == sb.samples
    o32, s32, _ = c.oracle(32)
    np.testing.assert_array_equal(_bits(a), _bits(o32))
    assert (a[..., 3] > 0).mean() > 0.02
