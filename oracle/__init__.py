"""CPU oracle for the single-volume ray march -- TEST INFRASTRUCTURE ONLY.

ctypes bindings over ``oracle/_build/liborc.so`` (oracle/cpu_raycaster.cpp),
a C++ restatement of Voreen's CPURaycaster path plus the GLSL-only shading,
MIP and ISO rules. Only tests, the smoke check and the benchmark's CPU
baseline use it, to compare results with; the product library never does.

Parity status: the trilinear interpolation / normalisation and the camera
matrices are pinned against the reference's own compiled code (golden
vectors in tests/golden, made by tests/golden/make_golden.py through
oracle/_ref). The TF bake and the march loop follow the cited reference
lines but have no reference-produced golden outputs (parity unpinned for
those parts).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

U8, U16, F32 = 0, 1, 2
DVR, MIP, ISO, MOP, MIDA, FHP, FHN = 0, 1, 2, 3, 4, 5, 6
SHADE_NONE, SHADE_PHONG = 0, 1
_DT = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32}


class OrcVolume(C.Structure):
    _fields_ = [("data", C.c_void_p), ("dtype", C.c_int), ("dims", C.c_int * 3), ("spacing", C.c_float * 3),
                ("offset", C.c_float * 3), ("rwm_scale", C.c_float), ("rwm_offset", C.c_float)]


class OrcTF(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("width", C.c_int), ("domain_lo", C.c_float), ("domain_hi", C.c_float)]


class OrcParams(C.Structure):
    _fields_ = [("sampling_rate", C.c_float), ("compositing", C.c_int), ("shading", C.c_int),
                ("iso_value", C.c_float), ("ert_threshold", C.c_float), ("light_pos_phys", C.c_float * 3),
                ("camera_pos_phys", C.c_float * 3), ("light_ambient", C.c_float * 3),
                ("light_diffuse", C.c_float * 3), ("light_specular", C.c_float * 3), ("shininess", C.c_float),
                ("apply_attenuation", C.c_int), ("attenuation", C.c_float * 3), ("mida_gamma", C.c_float),
                ("preint", C.c_void_p), ("preint_res", C.c_int)]


class OrcTFKey(C.Structure):
    _fields_ = [("intensity", C.c_float), ("color_l", C.c_uint8 * 4), ("color_r", C.c_uint8 * 4)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.POINTER
        L.oracle_bake_tf_keys.argtypes = [P(OrcTFKey), C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_void_p]
        L.oracle_preint_source.argtypes = [P(OrcTFKey), C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                           C.c_void_p]
        L.oracle_preint_table.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_int, C.c_void_p]
        L.oracle_entry_exit.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.oracle_entry_exit_box.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p]
        for name in ("oracle_render_f32", "oracle_render_f64"):
            getattr(L, name).argtypes = [P(OrcVolume), P(OrcTF), P(OrcParams), C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
        L.oracle_trilinear_f32.argtypes = [P(OrcVolume), C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_brick_minmax.argtypes = [P(OrcVolume), C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def make_volume(vox: np.ndarray, spacing=(1, 1, 1), offset=(0, 0, 0), rwm=(1.0, 0.0)) -> OrcVolume:
    """vox: (Z, Y, X) C-contiguous uint8/uint16/float32."""
    assert vox.flags.c_contiguous and vox.ndim == 3
    v = OrcVolume()
    v.data = vox.ctypes.data
    v.dtype = _DT[vox.dtype]
    v.dims[:] = [vox.shape[2], vox.shape[1], vox.shape[0]]
    v.spacing[:] = list(spacing)
    v.offset[:] = list(offset)
    v.rwm_scale, v.rwm_offset = rwm
    v._keep = vox
    return v


def make_params(sampling_rate=2.0, compositing=DVR, shading=SHADE_NONE, iso_value=0.5, ert=0.95,
                light_pos=(2.3, 1.5, 1.5), camera_pos=(0, 0, 3), ambient=(0.4,) * 3, diffuse=(0.8,) * 3,
                specular=(0.6,) * 3, shininess=60.0, attenuation=None, mida_gamma=0.0,
                preint_table: np.ndarray | None = None) -> OrcParams:
    """preint_table: (res, res, 4) float32 pre-integration table ([back, front]),
    None = classification by the TF."""
    p = OrcParams()
    p.mida_gamma = mida_gamma
    if preint_table is not None:
        t = np.ascontiguousarray(preint_table, dtype=np.float32)
        assert t.ndim == 3 and t.shape[0] == t.shape[1] and t.shape[2] == 4
        p.preint = t.ctypes.data
        p.preint_res = t.shape[0]
        p._keep = t
    p.sampling_rate = sampling_rate
    p.compositing = compositing
    p.shading = shading
    p.iso_value = iso_value
    p.ert_threshold = ert
    p.light_pos_phys[:] = list(light_pos)[:3]
    p.camera_pos_phys[:] = list(camera_pos)[:3]
    p.light_ambient[:] = list(ambient)
    p.light_diffuse[:] = list(diffuse)
    p.light_specular[:] = list(specular)
    p.shininess = shininess
    p.apply_attenuation = 1 if attenuation is not None else 0
    p.attenuation[:] = list(attenuation) if attenuation is not None else [1.0, 0.0, 0.0]
    return p


def bake_tf(keys, width, gamma=1.0, threshold=(0.0, 1.0)) -> np.ndarray:
    """keys: list of (intensity, (r,g,b,a)) or (intensity, colorL, colorR)."""
    arr = (OrcTFKey * max(1, len(keys)))()
    for i, k in enumerate(keys):
        arr[i].intensity = k[0]
        arr[i].color_l[:] = list(k[1])
        arr[i].color_r[:] = list(k[2] if len(k) > 2 else k[1])
    out = np.zeros((width, 4), np.uint8)
    lib().oracle_bake_tf_keys(arr, len(keys), width, gamma, threshold[0], threshold[1], _ptr(out))
    return out


def _keys(keys):
    arr = (OrcTFKey * max(1, len(keys)))()
    for i, k in enumerate(keys):
        arr[i].intensity = k[0]
        arr[i].color_l[:] = list(k[1])
        arr[i].color_r[:] = list(k[2] if len(k) > 2 else k[1])
    return arr


def preint_source(keys, res, gamma=1.0, threshold=(0.0, 1.0)) -> np.ndarray:
    """The TF sampled at `res` entries as the pre-integration table build does."""
    out = np.zeros((res, 4), np.uint8)
    lib().oracle_preint_source(_keys(keys), len(keys), res, gamma, threshold[0], threshold[1], _ptr(out))
    return out


def preint_table(source_rgba: np.ndarray, step: float, use_integral: bool = False) -> np.ndarray:
    """(res, res, 4) float32 table, [back, front] (PreIntegrationTable::computeTable)."""
    src = np.ascontiguousarray(source_rgba, dtype=np.uint8)
    res = src.shape[0]
    out = np.zeros((res, res, 4), np.float32)
    lib().oracle_preint_table(_ptr(src), res, step, 1 if use_integral else 0, _ptr(out))
    return out


def entry_exit(inv_mvp: np.ndarray, width: int, height: int, quantize16: bool = False, box=None):
    """box: ((lo x, y, z), (hi x, y, z)) texture-space clip box, None = the unit cube."""
    m = np.ascontiguousarray(inv_mvp, dtype=np.float64)
    e = np.zeros((height, width, 4), np.float32)
    x = np.zeros((height, width, 4), np.float32)
    if box is None:
        lib().oracle_entry_exit(_ptr(m), width, height, 1 if quantize16 else 0, _ptr(e), _ptr(x))
    else:
        lo = np.ascontiguousarray(box[0], dtype=np.float64)
        hi = np.ascontiguousarray(box[1], dtype=np.float64)
        lib().oracle_entry_exit_box(_ptr(m), width, height, 1 if quantize16 else 0, _ptr(lo), _ptr(hi), _ptr(e),
                                    _ptr(x))
    return e, x


def render(vol: OrcVolume, tf_rgba: np.ndarray, domain, params: OrcParams, entry: np.ndarray, exit_pts: np.ndarray,
           precision: int = 32, rows=None, nthreads: int = 0, signature: np.ndarray | None = None):
    """Returns (rgba (H,W,4), samples (H,W) int32, first_hit (H,W)).
    signature: optional (H, W) uint32 array that receives each ray's decision
    signature (a hash of the TF entries with alpha > 0 it picked, by sample)."""
    H, W = entry.shape[:2]
    tf_rgba = np.ascontiguousarray(tf_rgba, dtype=np.uint8)
    tf = OrcTF()
    tf.rgba = tf_rgba.ctypes.data
    tf.width = tf_rgba.shape[0]
    tf.domain_lo, tf.domain_hi = domain
    e = np.ascontiguousarray(entry, dtype=np.float32)
    x = np.ascontiguousarray(exit_pts, dtype=np.float32)
    ft = np.float32 if precision == 32 else np.float64
    out = np.zeros((H, W, 4), ft)
    samples = np.zeros((H, W), np.int32)
    fh = np.full((H, W), -1, ft)
    r0, r1 = (0, H) if rows is None else rows
    fn = lib().oracle_render_f32 if precision == 32 else lib().oracle_render_f64
    if signature is not None:
        assert signature.dtype == np.uint32 and signature.shape == (H, W) and signature.flags.c_contiguous
    fn(C.byref(vol), C.byref(tf), C.byref(params), _ptr(e), _ptr(x), W, H, r0, r1, nthreads, _ptr(out),
       _ptr(samples), _ptr(fh), _ptr(signature) if signature is not None else None)
    return out, samples, fh


def trilinear(vol: OrcVolume, pos: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    out = np.zeros(len(p), np.float32)
    lib().oracle_trilinear_f32(C.byref(vol), _ptr(p), len(p), _ptr(out))
    return out


def brick_minmax(vol: OrcVolume, brick: int, apron_hi: int = 1):
    nb = [(vol.dims[i] + brick - 1) // brick for i in range(3)]
    mn = np.zeros(nb[0] * nb[1] * nb[2], np.float32)
    mx = np.zeros_like(mn)
    lib().oracle_brick_minmax(C.byref(vol), brick, apron_hi, _ptr(mn), _ptr(mx))
    return mn, mx, nb


def half_sample_mean(vox: np.ndarray) -> np.ndarray:
    """Half-resolution level of a (Z, Y, X) volume: each voxel the mean of the
    2x2x2 block at twice its index, indices clamped to the volume. Integers
    follow HalfSampleMean (src/core/datastructures/octree/volumeoctree.cpp:
    188-202): exact sum, divided by 8 with truncation; floats are summed in
    z, y, x order in float32 and scaled by 1/8."""
    d = vox.shape
    d1 = tuple((n + 1) // 2 for n in d)
    idx = [np.minimum(2 * np.arange(d1[a])[:, None] + np.arange(2)[None, :], d[a] - 1) for a in range(3)]
    if vox.dtype == np.float32:
        acc = np.zeros(d1, np.float32)
        for dz in range(2):
            for dy in range(2):
                for dx in range(2):
                    acc = acc + vox[np.ix_(idx[0][:, dz], idx[1][:, dy], idx[2][:, dx])]
        return (acc * np.float32(0.125)).astype(np.float32)
    acc = np.zeros(d1, np.uint64)
    for dz in range(2):
        for dy in range(2):
            for dx in range(2):
                acc += vox[np.ix_(idx[0][:, dz], idx[1][:, dy], idx[2][:, dx])].astype(np.uint64)
    return (acc // 8).astype(vox.dtype)


_synth = None


def synth_volume(kind: int, dtype: int, dims_xyz, seed: int) -> np.ndarray:
    """The seeded workload volume (the same generator source as the product's
    vrc_synth_volume, built as oracle/_build/libsynth.so), (Z, Y, X)."""
    global _synth
    if _synth is None:
        _synth = C.CDLL(_build.build_synth())
        _synth.vrc_synth_volume.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.c_uint64, C.c_void_p]
        _synth.vrc_synth_volume.restype = C.c_int
    X, Y, Z = dims_xyz
    out = np.empty((Z, Y, X), {U8: np.uint8, U16: np.uint16, F32: np.float32}[dtype])
    if _synth.vrc_synth_volume(kind, dtype, (C.c_int * 3)(X, Y, Z), seed, _ptr(out)) != 0:
        raise ValueError("vrc_synth_volume: invalid arguments")
    return out


# ---- the reference pin library (present only where the reference tree is) ----
_ref = None


def ref_lib(reference_root: str | None = None):
    """The reference's own VolumeRAM trilinear + tgt math, or None."""
    global _ref
    if _ref is None:
        path = _build.build_ref(reference_root or _build.DEFAULT_REFERENCE)
        if path is None:
            if os.path.exists(_build.REF_LIB):
                path = _build.REF_LIB
            else:
                return None
        L = C.CDLL(path)
        L.ref_trilinear.argtypes = [C.c_int, C.c_void_p, C.POINTER(C.c_int), C.c_void_p, C.c_int, C.c_void_p]
        L.ref_lookat.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_perspective.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p]
        L.ref_iround.argtypes = [C.c_float]
        L.ref_iround.restype = C.c_int
        _ref = L
    return _ref


_ref_tf = None


def ref_tf_lib(reference_root: str | None = None):
    """The reference's own TF bake arithmetic (oracle/_ref/libvoreen_tf_ref.so), or None."""
    global _ref_tf
    if _ref_tf is None:
        path = _build.build_tf_ref(reference_root or _build.DEFAULT_REFERENCE)
        if path is None:
            if os.path.exists(_build.REF_TF_LIB):
                path = _build.REF_TF_LIB
            else:
                return None
        L = C.CDLL(path)
        L.ref_tf_bake.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                  C.c_void_p]
        _ref_tf = L
    return _ref_tf


def ref_bake_tf(keys, width, gamma=1.0, threshold=(0.0, 1.0), reference_root: str | None = None):
    """The TF table as the reference's own code bakes it (None without the
    reference tree). keys as for bake_tf."""
    L = ref_tf_lib(reference_root)
    if L is None:
        return None
    inten = np.array([k[0] for k in keys] or [0.0], np.float32)
    cols = np.array([list(k[1]) + list(k[2] if len(k) > 2 else k[1]) for k in keys] or [[0] * 8], np.uint8)
    out = np.zeros((width, 4), np.uint8)
    L.ref_tf_bake(_ptr(inten), _ptr(cols), len(keys), width, gamma, threshold[0], threshold[1], _ptr(out))
    return out
