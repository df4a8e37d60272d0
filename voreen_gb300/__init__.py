"""voreen_gb300 -- a GB300-native single-volume raycaster.

Python view of the C ABI (include/vrc.h). The compute path is the in-tree
CUDA library ``_build/libvrc.so``; there is no CPU fallback, and every call
raises ``VrcError`` when the library reports a failure.

Typical use (mirrors Voreen's CPURaycaster processor; see ``raycaster``)::

    ctx = Context()
    vol = Volume(ctx, voxels_zyx, spacing=(0.7, 0.7, 1.0))
    tf = TransferFunction(ctx, TransferFunction.bake(keys, 4096), domain=(lo, hi))
    p = default_params(1920, 1080)
    img, stats = render(ctx, vol, tf, p, entry, exit_pts)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import (CLASSIFY_PREINTEGRATED, CLASSIFY_TF, DVR, EE_ANALYTIC, EE_BUFFERS, F32, FHN, FHP, ISO, MIDA, MIP,
                   MOP, NOALLOC_MAX_CELLS, PLACE_DEVICE, PLACE_HOST, OUT_RGBA8, OUT_RGBA16, OUT_RGBA32F, SHADE_NONE, SHADE_PHONG, U8, U16,
                   Camera, RenderParams, RenderStats, TFKey, VolumeDesc)

__all__ = ["VrcError", "Context", "Volume", "TransferFunction", "PreIntegrationTable", "render", "entry_exit",
           "default_params", "sampling_step", "image_rescale", "read_vvd_header", "write_vvd", "camera_matrices", "lib", "DVR", "MIP", "ISO", "MOP", "MIDA", "FHP",
           "FHN", "CLASSIFY_TF", "CLASSIFY_PREINTEGRATED", "SHADE_NONE", "SHADE_PHONG", "U8", "U16", "F32",
           "OUT_RGBA8", "OUT_RGBA16", "OUT_RGBA32F", "EE_BUFFERS", "EE_ANALYTIC", "Camera", "RenderParams",
           "RenderStats", "VolumeDesc", "TFKey"]

_NP_DTYPE = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32}
_DTYPE_NP = {U8: np.uint8, U16: np.uint16, F32: np.float32}


def lib():
    """The loaded libvrc.so with its ctypes signatures (raises when it is not built)."""
    return _abi.load()


class VrcError(RuntimeError):
    """A vrc_status other than VRC_OK, with the context's error detail; `status`
    holds the code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _check(status: int, ctx=None, what: str = ""):
    if status != _abi.VRC_OK:
        detail = ""
        if ctx is not None and ctx.handle:
            detail = (lib().vrc_last_error(ctx.handle) or b"").decode()
        raise VrcError(status, f"{what}: {detail}" if detail else what)


def _is_device(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _ptr(a):
    if a is None:
        return None
    if _is_device(a):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One CUDA device and stream (vrc_context)."""

    def __init__(self, device: int = 0):
        self.handle = C.c_void_p()
        _check(lib().vrc_context_create(device, C.byref(self.handle)), None, "vrc_context_create")
        self.device = device

    @property
    def stream(self) -> int:
        return lib().vrc_context_stream(self.handle) or 0

    def synchronize(self):
        _check(lib().vrc_context_synchronize(self.handle), self, "vrc_context_synchronize")

    def close(self):
        if self.handle:
            lib().vrc_context_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_desc(dtype: int, dims_xyz, spacing=(1.0, 1.0, 1.0), offset=(0.0, 0.0, 0.0), rwm=(1.0, 0.0)) -> VolumeDesc:
    """vrc_volume_desc: dtype, dims (x, y, z), spacing, offset and the real-world
    mapping (scale, offset) of a volume."""
    d = VolumeDesc()
    d.dtype = dtype
    d.dims[:] = [int(v) for v in dims_xyz]
    d.spacing[:] = [float(v) for v in spacing]
    d.offset[:] = [float(v) for v in offset]
    d.rwm_scale, d.rwm_offset = float(rwm[0]), float(rwm[1])
    return d


class Volume:
    """A volume in the bricked device layout (vrc_volume).

    ``voxels``: numpy (Z, Y, X) array (x fastest, VolumeAtomic::calcPos) of
    uint8 / uint16 / float32, or a CUDA tensor of the same layout.
    """

    def __init__(self, ctx: Context, voxels, spacing=(1.0, 1.0, 1.0), offset=(0.0, 0.0, 0.0), rwm=(1.0, 0.0),
                 brick_size: int = 0, placement: int = 0):
        self.ctx = ctx
        if _is_device(voxels):
            import torch
            dt = {torch.uint8: U8, torch.uint16: U16, torch.float32: F32}[voxels.dtype]
            assert voxels.is_contiguous() and voxels.dim() == 3
            shape = tuple(voxels.shape)
        else:
            voxels = np.ascontiguousarray(voxels)
            dt = _NP_DTYPE[voxels.dtype]
            shape = voxels.shape
        self.desc = make_desc(dt, (shape[2], shape[1], shape[0]), spacing, offset, rwm)
        self.placement = placement
        self.handle = C.c_void_p()
        _check(lib().vrc_volume_upload_placed(ctx.handle, C.byref(self.desc), _ptr(voxels),
                                              1 if _is_device(voxels) else 0, brick_size, placement,
                                              C.byref(self.handle)), ctx, "vrc_volume_upload")

    @classmethod
    def load_vvd(cls, ctx: Context, path: str, brick_size: int = 0) -> "Volume":
        """A Voreen .vvd volume file straight into the bricked device layout
        (vrc_volume_load_vvd); the header is in `.vvd_info`."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.placement = PLACE_DEVICE
        self.handle = C.c_void_p()
        info = _abi.VvdInfo()
        _check(lib().vrc_volume_load_vvd(ctx.handle, path.encode(), brick_size, C.byref(self.handle), C.byref(info)),
               ctx, "vrc_volume_load_vvd")
        self.vvd_info = info
        self.desc = make_desc(info.dtype, tuple(info.dims), tuple(info.spacing), tuple(info.offset),
                              (info.rwm_scale, info.rwm_offset))
        return self

    @property
    def dims(self):
        return tuple(self.desc.dims)

    @property
    def dtype(self) -> int:
        return self.desc.dtype

    def minmax(self):
        a, b = C.c_float(), C.c_float()
        _check(lib().vrc_volume_minmax(self.handle, C.byref(a), C.byref(b)), self.ctx, "vrc_volume_minmax")
        return a.value, b.value

    def brick_minmax(self):
        nb = (C.c_int * 3)()
        _check(lib().vrc_volume_brick_minmax(self.handle, nb, None, None), self.ctx, "vrc_volume_brick_minmax")
        n = nb[0] * nb[1] * nb[2]
        mn = np.zeros(n, np.float32)
        mx = np.zeros(n, np.float32)
        _check(lib().vrc_volume_brick_minmax(self.handle, nb, _ptr(mn), _ptr(mx)), self.ctx, "vrc_volume_brick_minmax")
        return mn, mx, tuple(nb)

    @property
    def device_bytes(self) -> int:
        return int(lib().vrc_volume_device_bytes(self.handle))

    @property
    def host_bytes(self) -> int:
        return int(lib().vrc_volume_host_bytes(self.handle))

    def set_cache_limit(self, nbytes: int):
        """Device brick cache budget of a host-placed pool (0 = read the host
        pool only; the default is bounded by free device memory)."""
        _check(lib().vrc_volume_set_cache_limit(self.handle, int(nbytes)), self.ctx, "vrc_volume_set_cache_limit")

    def cache_info(self):
        """(bricks cached, bricks the last TF could reach, bricks the last
        tracked render read without a cache slot)."""
        c, r, m = C.c_longlong(0), C.c_longlong(0), C.c_longlong(0)
        _check(lib().vrc_volume_cache_info(self.handle, C.byref(c), C.byref(r), C.byref(m)), self.ctx,
               "vrc_volume_cache_info")
        return int(c.value), int(r.value), int(m.value)

    def set_cache_upload_budget(self, nbytes: int):
        """Bytes of bricks gathered into the device cache per render (0 = unlimited)."""
        _check(lib().vrc_volume_set_cache_upload_budget(self.handle, int(nbytes)), self.ctx,
               "vrc_volume_set_cache_upload_budget")

    def set_lod(self, level=True):
        """Sample bricks without a cache slot from a device-resident coarser
        level (host-placed pools only): True or 1 = half resolution, k = the
        level 2^-k of the 2x2x2-mean pyramid, False or 0 = off."""
        k = int(level) if not isinstance(level, bool) else (1 if level else 0)
        _check(lib().vrc_volume_set_lod(self.handle, k), self.ctx, "vrc_volume_set_lod")

    def close(self):
        if self.handle:
            lib().vrc_volume_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TransferFunction:
    """A baked RGBA8 1D transfer function with its real-world domain (vrc_tf)."""

    def __init__(self, ctx: Context, rgba: np.ndarray, domain=(0.0, 1.0)):
        self.ctx = ctx
        self.rgba = np.ascontiguousarray(rgba, dtype=np.uint8).reshape(-1, 4)
        self.domain = (float(domain[0]), float(domain[1]))
        self.handle = C.c_void_p()
        _check(lib().vrc_tf_create(ctx.handle, _ptr(self.rgba), self.rgba.shape[0], self.domain[0], self.domain[1],
                                   C.byref(self.handle)), ctx, "vrc_tf_create")

    @staticmethod
    def bake(keys, width: int, gamma: float = 1.0, threshold=(0.0, 1.0)) -> np.ndarray:
        """Host-only TransFunc1DKeys bake. keys: [(intensity, rgba) or (intensity, rgbaL, rgbaR)]."""
        arr = (TFKey * max(1, len(keys)))()
        for i, k in enumerate(keys):
            arr[i].intensity = float(k[0])
            arr[i].color_l[:] = [int(v) for v in k[1]]
            arr[i].color_r[:] = [int(v) for v in (k[2] if len(k) > 2 else k[1])]
        out = np.zeros((width, 4), np.uint8)
        _check(lib().vrc_tf_bake_keys(arr, len(keys), width, gamma, threshold[0], threshold[1], _ptr(out)), None,
               "vrc_tf_bake_keys")
        return out

    @staticmethod
    def table_width(dtype: int) -> int:
        return int(lib().vrc_tf_table_width(dtype))

    def set_preintegration(self, table: "PreIntegrationTable | None"):
        """Attach (or with None detach) the table used by renders with
        classification CLASSIFY_PREINTEGRATED."""
        _check(lib().vrc_tf_set_preintegration(self.handle, table.handle if table is not None else None), self.ctx,
               "vrc_tf_set_preintegration")
        self._preint = table

    def close(self):
        if self.handle:
            lib().vrc_tf_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _tf_keys(keys):
    arr = (TFKey * max(1, len(keys)))()
    for i, k in enumerate(keys):
        arr[i].intensity = float(k[0])
        arr[i].color_l[:] = [int(v) for v in k[1]]
        arr[i].color_r[:] = [int(v) for v in (k[2] if len(k) > 2 else k[1])]
    return arr


class PreIntegrationTable:
    """Pre-integrated classification table on the device (vrc_preint,
    PreIntegrationTable): res x res RGBA, entry [back, front], for one
    sampling step size."""

    def __init__(self, ctx: Context, source_rgba: np.ndarray, step: float, use_integral: bool = False):
        self.ctx = ctx
        self.source = np.ascontiguousarray(source_rgba, dtype=np.uint8).reshape(-1, 4)
        self.res = self.source.shape[0]
        self.step = float(np.float32(step))
        self.use_integral = bool(use_integral)
        self.handle = C.c_void_p()
        _check(lib().vrc_preint_create(ctx.handle, _ptr(self.source), self.res, self.step, 1 if use_integral else 0,
                                       C.byref(self.handle)), ctx, "vrc_preint_create")

    @staticmethod
    def resolution(tf_width: int, requested: int = 0) -> int:
        return int(lib().vrc_preint_resolution(tf_width, requested))

    @staticmethod
    def bake_source(keys, res: int, gamma: float = 1.0, threshold=(0.0, 1.0)) -> np.ndarray:
        """The TF keys sampled at `res` entries as the table build samples them."""
        out = np.zeros((res, 4), np.uint8)
        _check(lib().vrc_preint_bake_source(_tf_keys(keys), len(keys), res, gamma, threshold[0], threshold[1],
                                            _ptr(out)), None, "vrc_preint_bake_source")
        return out

    def download(self) -> np.ndarray:
        out = np.zeros((self.res, self.res, 4), np.float32)
        _check(lib().vrc_preint_download(self.handle, _ptr(out)), self.ctx, "vrc_preint_download")
        return out

    def close(self):
        if self.handle:
            lib().vrc_preint_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_vvd_header(path: str):
    """vrc_vvd_read_header: the parsed .vvd header (VvdInfo)."""
    info = _abi.VvdInfo()
    _check(lib().vrc_vvd_read_header(path.encode(), C.byref(info)), None, "vrc_vvd_read_header")
    return info


def write_vvd(path: str, voxels: np.ndarray, spacing=(1.0, 1.0, 1.0), offset=(0.0, 0.0, 0.0), rwm=None,
              path_list: bool = False):
    """Write (Z, Y, X) voxels as <path>.raw plus a .vvd header in Voreen's
    layout (RawData with a `filename` attribute, or with the path list of
    newer files). For tests and benchmarks; the product reads, it does not
    need to write."""
    import os
    voxels = np.ascontiguousarray(voxels)
    fmt = {np.dtype(np.uint8): "uint8", np.dtype(np.uint16): "uint16", np.dtype(np.float32): "float"}[voxels.dtype]
    raw = os.path.splitext(path)[0] + ".raw"
    voxels.tofile(raw)
    Z, Y, X = voxels.shape
    name = os.path.basename(raw)
    if path_list:
        rawdata = (f'<RawData format="{fmt}" x="{X}" y="{Y}" z="{Z}">\n'
                   f'                <Paths noPathSet="false">\n                    <paths>\n'
                   f'                        <item value="missing/{name}" />\n'
                   f'                        <item value="{name}" />\n'
                   f'                    </paths>\n                </Paths>\n            </RawData>')
    else:
        rawdata = f'<RawData filename="{name}" format="{fmt}" x="{X}" y="{Y}" z="{Z}" />'
    meta = (f'                <MetaItem name="Offset" type="Vec3MetaData">\n'
            f'                    <value x="{offset[0]!r}" y="{offset[1]!r}" z="{offset[2]!r}" />\n'
            f'                </MetaItem>\n'
            f'                <MetaItem name="Spacing" type="Vec3MetaData">\n'
            f'                    <value x="{spacing[0]!r}" y="{spacing[1]!r}" z="{spacing[2]!r}" />\n'
            f'                </MetaItem>\n')
    if rwm is not None:
        meta += (f'                <MetaItem name="RealWorldMapping" type="RealWorldMappingMetaData">\n'
                 f'                    <value scale="{rwm[0]!r}" offset="{rwm[1]!r}" unit="" />\n'
                 f'                </MetaItem>\n')
    with open(path, "w") as f:
        f.write('<?xml version="1.0" ?>\n<VoreenData version="1">\n    <Volumes>\n        <Volume>\n'
                f'            {rawdata}\n            <MetaData>\n{meta}            </MetaData>\n'
                '        </Volume>\n    </Volumes>\n</VoreenData>\n')
    return raw


def image_rescale(ctx: Context, src, dst, out_format: int = OUT_RGBA32F):
    """Bilinear rescale (GL_LINEAR, clamp to edge) of the device RGBA image
    `src` (h, w, 4) into `dst` (H, W, 4), on the context stream."""
    h, w = src.shape[0], src.shape[1]
    H, W = dst.shape[0], dst.shape[1]
    _check(lib().vrc_image_rescale(ctx.handle, _ptr(src), w, h, _ptr(dst), W, H, out_format), ctx,
           "vrc_image_rescale")


def sampling_step(vol: "Volume", sampling_rate: float) -> float:
    """The march's step size 1 / (max(dim) * samplingRate) in FP32."""
    return float(lib().vrc_sampling_step(vol.handle, sampling_rate))


def read_tfi(path: str) -> dict:
    """A Voreen .tfi transfer function (vrc_tf_read_tfi): keys as
    (intensity, colorL, colorR), gamma, thresholds, domain, width, alphaMode."""
    info = _abi.TfiInfo()
    _check(lib().vrc_tf_read_tfi(path.encode(), C.byref(info), None, 0), None, "vrc_tf_read_tfi")
    keys = (TFKey * max(1, info.nkeys))()
    _check(lib().vrc_tf_read_tfi(path.encode(), C.byref(info), keys, info.nkeys), None, "vrc_tf_read_tfi")
    return {"keys": [(float(k.intensity), tuple(k.color_l), tuple(k.color_r)) for k in keys[:info.nkeys]],
            "gamma": float(info.gamma), "threshold": (float(info.threshold[0]), float(info.threshold[1])),
            "domain": (float(info.domain[0]), float(info.domain[1])), "width": int(info.width),
            "alpha_mode": int(info.alpha_mode)}


def measure_l2_read(ctx: Context, nbytes: int = 48 << 20, reps: int = 40) -> float:
    """L2-resident read bandwidth in GB/s (vrc_measure_l2_read)."""
    g = C.c_float()
    _check(lib().vrc_measure_l2_read(ctx.handle, int(nbytes), int(reps), C.byref(g)), ctx, "vrc_measure_l2_read")
    return float(g.value)


def default_params(width: int, height: int) -> RenderParams:
    """Render parameters with the reference processor's property defaults
    (vrc_render_params_default) for a width x height image."""
    p = RenderParams()
    lib().vrc_render_params_default(C.byref(p), width, height)
    return p


def make_camera(position, focus, up=(0.0, 1.0, 0.0), fovy=45.0, near=0.1, far=50.0, ratio=1.0) -> Camera:
    """A perspective camera (tgt::Camera fields: position, focus, up, vertical
    field of view in degrees, near/far distances, frustum ratio)."""
    c = Camera()
    c.position[:] = [float(v) for v in position]
    c.focus[:] = [float(v) for v in focus]
    c.up[:] = [float(v) for v in up]
    c.fovy_deg, c.near_dist, c.far_dist, c.frustum_ratio = fovy, near, far, ratio
    return c


def camera_matrices(cam: Camera, desc: VolumeDesc, width: int, height: int):
    """(view, projection, inverse(projection * view * textureToWorld)) as
    4 x 4 float64 arrays, computed as the reference does (vrc_camera_matrices)."""
    v = np.zeros(16, np.float64)
    p = np.zeros(16, np.float64)
    inv = np.zeros(16, np.float64)
    _check(lib().vrc_camera_matrices(C.byref(cam), C.byref(desc), width, height, _ptr(v), _ptr(p), _ptr(inv)), None,
           "vrc_camera_matrices")
    return v.reshape(4, 4), p.reshape(4, 4), inv.reshape(4, 4)


_OUT_NP = {OUT_RGBA8: (np.uint8, 4), OUT_RGBA16: (np.uint16, 4), OUT_RGBA32F: (np.float32, 4)}


def render(ctx: Context, vol: Volume, tf: TransferFunction, params: RenderParams, entry=None, exit_pts=None,
           out_format: int = OUT_RGBA32F, out=None):
    """One frame. entry/exit: (H, W, 4) float32 host arrays or CUDA tensors
    (ignored in analytic mode). Returns (image, RenderStats); image is `out`
    if given (host array or CUDA tensor), else a new host array."""
    H, W = params.height, params.width
    if out is None:
        dt, ch = _OUT_NP[out_format]
        out = np.zeros((H, W, ch), dt)
    ee_dev = 1 if (entry is not None and _is_device(entry)) else 0
    if entry is not None and not ee_dev:
        entry = np.ascontiguousarray(entry, dtype=np.float32)
        exit_pts = np.ascontiguousarray(exit_pts, dtype=np.float32)
    stats = RenderStats()
    _check(lib().vrc_render(ctx.handle, vol.handle, tf.handle, C.byref(params), _ptr(entry), _ptr(exit_pts), ee_dev,
                            _ptr(out), out_format, 1 if _is_device(out) else 0, C.byref(stats)), ctx, "vrc_render")
    return out, stats


def render_async(ctx: Context, vol: Volume, tf: TransferFunction, params: RenderParams, entry, exit_pts, out,
                 out_format: int = OUT_RGBA32F):
    """Device-resident frame: enqueue only (no stats, no synchronize)."""
    ee_dev = 1 if (entry is not None and _is_device(entry)) else 0
    _check(lib().vrc_render(ctx.handle, vol.handle, tf.handle, C.byref(params), _ptr(entry), _ptr(exit_pts), ee_dev,
                            _ptr(out), out_format, 1, None), ctx, "vrc_render")


def render_noalloc(vol: Volume, tf: TransferFunction, params: RenderParams, entry, exit_pts, out,
                   out_format: int = OUT_RGBA32F, stream: int = 0):
    """vrc_render_noalloc: enqueue a frame on `stream` with no allocation.
    entry/exit/out are CUDA tensors (entry/exit may be None in analytic mode)."""
    st = lib().vrc_render_noalloc(vol.handle, tf.handle, C.byref(params), _ptr(entry), _ptr(exit_pts), _ptr(out),
                                  out_format, C.c_void_p(stream))
    _check(st, None, "vrc_render_noalloc")


class Batch:
    """Many requests in one persistent launch replayed from a captured CUDA
    graph (vrc_batch_*). items: [(Volume, TransferFunction, RenderParams,
    out CUDA tensor, out_format)]; params must use analytic entry/exit and
    share compositing and shading. Volume / TransferFunction may be None.
    isolate=True (vrc_batch_create_isolated): invalid requests are left out
    and `status` holds each request's vrc_status; otherwise any invalid
    request raises."""

    def __init__(self, ctx: Context, items, isolate: bool = False):
        self.ctx = ctx
        self.items = list(items)
        arr = (_abi.BatchItem * len(self.items))()
        for i, (vol, tf, p, out, fmt) in enumerate(self.items):
            arr[i].volume = vol.handle.value if vol is not None else None
            arr[i].tf = tf.handle.value if tf is not None else None
            arr[i].params = p
            arr[i].out = out.data_ptr() if out is not None else None
            arr[i].out_format = fmt
        self.handle = C.c_void_p()
        if isolate:
            st = (C.c_int * len(self.items))()
            _check(lib().vrc_batch_create_isolated(ctx.handle, arr, len(self.items), st, C.byref(self.handle)), ctx,
                   "vrc_batch_create_isolated")
            self.status = [int(x) for x in st]
        else:
            _check(lib().vrc_batch_create(ctx.handle, arr, len(self.items), C.byref(self.handle)), ctx,
                   "vrc_batch_create")
            self.status = [0] * len(self.items)

    def launch(self):
        _check(lib().vrc_batch_launch(self.handle), self.ctx, "vrc_batch_launch")

    def stats(self):
        lat = np.zeros(len(self.items), np.float32)
        st = _abi.BatchStats()
        _check(lib().vrc_batch_stats_get(self.handle, _ptr(lat), C.byref(st)), self.ctx, "vrc_batch_stats_get")
        return st, lat

    def close(self):
        if self.handle:
            lib().vrc_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def entry_exit(ctx: Context, vol: Volume, params: RenderParams):
    """Analytic entry/exit points for params.camera (host arrays)."""
    H, W = params.height, params.width
    e = np.zeros((H, W, 4), np.float32)
    x = np.zeros((H, W, 4), np.float32)
    _check(lib().vrc_entry_exit(ctx.handle, vol.handle, C.byref(params), _ptr(e), _ptr(x), 0), ctx, "vrc_entry_exit")
    return e, x


def synth_volume(kind: int, dtype: int, dims_xyz, seed: int) -> np.ndarray:
    """Seeded procedural volume (vrc_synth_volume), returned as (Z, Y, X)."""
    X, Y, Z = dims_xyz
    out = np.empty((Z, Y, X), _DTYPE_NP[dtype])
    d = (C.c_int * 3)(X, Y, Z)
    if lib().vrc_synth_volume(kind, dtype, d, seed, _ptr(out)) != 0:
        raise VrcError(1, "vrc_synth_volume: invalid arguments")
    return out


def synth_tubes_device(dims_xyz, ntubes: int, seed: int, noise_sigma: float = 10.0):
    """Seeded sparse tube volume generated on the GPU (vrc_synth_tubes_device),
    returned as a (Z, Y, X) uint16 CUDA tensor."""
    import torch
    X, Y, Z = dims_xyz
    out = torch.empty((Z, Y, X), dtype=torch.uint16, device="cuda")
    d = (C.c_int * 3)(X, Y, Z)
    st = lib().vrc_synth_tubes_device(C.c_void_p(out.data_ptr()), d, ntubes, seed, noise_sigma,
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if st != 0:
        raise VrcError(2 if st == 2 else 1, "vrc_synth_tubes_device failed")
    return out
