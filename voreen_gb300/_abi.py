"""ctypes view of the C ABI in include/vrc.h and include/vrc_synth.h.

The shared library is the in-tree build ``voreen_gb300/_build/libvrc.so``.
There is no fallback: if it is missing or cannot be loaded, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvrc.so")

VRC_OK = 0
STATUS_NAMES = {0: "VRC_OK", 1: "VRC_ERR_INVALID_ARG", 2: "VRC_ERR_CUDA", 3: "VRC_ERR_OUT_OF_MEMORY",
                4: "VRC_ERR_UNSUPPORTED", 5: "VRC_ERR_TIMEOUT", 6: "VRC_ERR_NOT_READY", 7: "VRC_ERR_DEVICE",
                8: "VRC_ERR_SCRATCH_LIMIT"}
U8, U16, F32 = 0, 1, 2
DVR, MIP, ISO, MOP, MIDA, FHP, FHN = 0, 1, 2, 3, 4, 5, 6
CLASSIFY_TF, CLASSIFY_PREINTEGRATED = 0, 1
SHADE_NONE, SHADE_PHONG = 0, 1
OUT_RGBA8, OUT_RGBA32F, OUT_RGBA16 = 0, 1, 2
EE_BUFFERS, EE_ANALYTIC = 0, 1
PLACE_DEVICE, PLACE_HOST = 0, 1
NOALLOC_MAX_CELLS = 2097152


class VolumeDesc(C.Structure):
    _fields_ = [("dtype", C.c_int), ("dims", C.c_int * 3), ("spacing", C.c_float * 3), ("offset", C.c_float * 3),
                ("rwm_scale", C.c_float), ("rwm_offset", C.c_float)]


class VvdInfo(C.Structure):
    _fields_ = [("dtype", C.c_int), ("dims", C.c_int * 3), ("spacing", C.c_float * 3), ("offset", C.c_float * 3),
                ("rwm_scale", C.c_float), ("rwm_offset", C.c_float), ("has_minmax", C.c_int),
                ("min_norm", C.c_float), ("max_norm", C.c_float), ("raw_path", C.c_char * 4096)]


class TFKey(C.Structure):
    _fields_ = [("intensity", C.c_float), ("color_l", C.c_uint8 * 4), ("color_r", C.c_uint8 * 4)]


class TfiInfo(C.Structure):
    _fields_ = [("width", C.c_int), ("alpha_mode", C.c_int), ("gamma", C.c_float), ("domain", C.c_float * 2),
                ("threshold", C.c_float * 2), ("nkeys", C.c_int)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("focus", C.c_float * 3), ("up", C.c_float * 3),
                ("fovy_deg", C.c_float), ("near_dist", C.c_float), ("far_dist", C.c_float),
                ("frustum_ratio", C.c_float)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("sampling_rate", C.c_float), ("compositing", C.c_int),
                ("shading", C.c_int), ("iso_value", C.c_float), ("ert_threshold", C.c_float),
                ("light_position", C.c_float * 4), ("light_ambient", C.c_float * 3),
                ("light_diffuse", C.c_float * 3), ("light_specular", C.c_float * 3),
                ("material_shininess", C.c_float), ("apply_attenuation", C.c_int),
                ("light_attenuation", C.c_float * 3), ("camera", Camera), ("entry_exit_mode", C.c_int),
                ("quantize_entry_exit", C.c_int), ("empty_space_skipping", C.c_int), ("skip_cell_size", C.c_int),
                ("tile_width", C.c_int), ("region", C.c_int * 4), ("classification", C.c_int),
                ("mida_gamma", C.c_float), ("enable_clipping", C.c_int), ("clip_llf", C.c_int * 3),
                ("clip_urb", C.c_int * 3)]


class BatchItem(C.Structure):
    _fields_ = [("volume", C.c_void_p), ("tf", C.c_void_p), ("params", RenderParams), ("out", C.c_void_p),
                ("out_format", C.c_int)]


class BatchStats(C.Structure):
    _fields_ = [("samples", C.c_double), ("total_ms", C.c_float), ("latency_p50_ms", C.c_float),
                ("latency_p99_ms", C.c_float), ("latency_max_ms", C.c_float),
                ("kernels_per_launch", C.c_int)]


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_double), ("samples_fetched", C.c_double), ("samples_shaded", C.c_double),
                ("skip_runs", C.c_double),
                ("kernel_ms", C.c_float), ("total_ms", C.c_float), ("device_status", C.c_int),
                ("kernel_launches", C.c_int)]


# name -> (restype, argtypes); every symbol declared in include/*.h
P = C.POINTER
VP = C.c_void_p
SIGNATURES = {
    "vrc_abi_version": (C.c_int, []),
    "vrc_status_string": (C.c_char_p, [C.c_int]),
    "vrc_last_error": (C.c_char_p, [VP]),
    "vrc_context_create": (C.c_int, [C.c_int, P(VP)]),
    "vrc_context_destroy": (C.c_int, [VP]),
    "vrc_context_synchronize": (C.c_int, [VP]),
    "vrc_context_stream": (VP, [VP]),
    "vrc_volume_upload": (C.c_int, [VP, P(VolumeDesc), VP, C.c_int, C.c_int, P(VP)]),
    "vrc_volume_destroy": (C.c_int, [VP]),
    "vrc_volume_upload_placed": (C.c_int, [VP, P(VolumeDesc), VP, C.c_int, C.c_int, C.c_int, P(VP)]),
    "vrc_volume_host_bytes": (C.c_size_t, [VP]),
    "vrc_volume_set_cache_limit": (C.c_int, [VP, C.c_size_t]),
    "vrc_volume_cache_info": (C.c_int, [VP, P(C.c_longlong), P(C.c_longlong), P(C.c_longlong)]),
    "vrc_volume_set_lod": (C.c_int, [VP, C.c_int]),
    "vrc_measure_l2_read": (C.c_int, [VP, C.c_size_t, C.c_int, P(C.c_float)]),
    "vrc_occupancy_distance": (C.c_int, [VP, VP, C.c_int, C.c_int, C.c_int, VP]),
    "vrc_tf_read_tfi": (C.c_int, [C.c_char_p, P(TfiInfo), P(TFKey), C.c_int]),
    "vrc_volume_set_cache_upload_budget": (C.c_int, [VP, C.c_size_t]),
    "vrc_volume_minmax": (C.c_int, [VP, P(C.c_float), P(C.c_float)]),
    "vrc_volume_brick_minmax": (C.c_int, [VP, P(C.c_int), VP, VP]),
    "vrc_volume_device_bytes": (C.c_size_t, [VP]),
    "vrc_tf_bake_keys": (C.c_int, [P(TFKey), C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, VP]),
    "vrc_tf_table_width": (C.c_int, [C.c_int]),
    "vrc_tf_create": (C.c_int, [VP, VP, C.c_int, C.c_float, C.c_float, P(VP)]),
    "vrc_tf_destroy": (C.c_int, [VP]),
    "vrc_camera_matrices": (C.c_int, [P(Camera), P(VolumeDesc), C.c_int, C.c_int, VP, VP, VP]),
    "vrc_render_params_default": (None, [P(RenderParams), C.c_int, C.c_int]),
    "vrc_render": (C.c_int, [VP, VP, VP, P(RenderParams), VP, VP, C.c_int, VP, C.c_int, C.c_int, P(RenderStats)]),
    "vrc_entry_exit": (C.c_int, [VP, VP, P(RenderParams), VP, VP, C.c_int]),
    "vrc_render_aux": (C.c_int, [VP, VP, VP, P(RenderParams), VP, VP, VP, C.c_int, VP, P(RenderStats)]),
    "vrc_batch_create": (C.c_int, [VP, P(BatchItem), C.c_int, P(VP)]),
    "vrc_batch_create_isolated": (C.c_int, [VP, P(BatchItem), C.c_int, P(C.c_int), P(VP)]),
    "vrc_batch_launch": (C.c_int, [VP]),
    "vrc_batch_stats_get": (C.c_int, [VP, VP, P(BatchStats)]),
    "vrc_batch_destroy": (C.c_int, [VP]),
    "vrc_render_noalloc": (C.c_int, [VP, VP, P(RenderParams), VP, VP, VP, C.c_int, VP]),
    "vrc_preint_resolution": (C.c_int, [C.c_int, C.c_int]),
    "vrc_preint_bake_source": (C.c_int, [P(TFKey), C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, VP]),
    "vrc_preint_create": (C.c_int, [VP, VP, C.c_int, C.c_float, C.c_int, P(VP)]),
    "vrc_preint_download": (C.c_int, [VP, VP]),
    "vrc_preint_destroy": (C.c_int, [VP]),
    "vrc_tf_set_preintegration": (C.c_int, [VP, VP]),
    "vrc_sampling_step": (C.c_float, [VP, C.c_float]),
    "vrc_vvd_read_header": (C.c_int, [C.c_char_p, P(VvdInfo)]),
    "vrc_volume_load_vvd": (C.c_int, [VP, C.c_char_p, C.c_int, P(VP), P(VvdInfo)]),
    "vrc_image_rescale": (C.c_int, [VP, VP, C.c_int, C.c_int, VP, C.c_int, C.c_int, C.c_int]),
    "vrc_synth_volume": (C.c_int, [C.c_int, C.c_int, P(C.c_int), C.c_uint64, VP]),
    "vrc_synth_tubes_device": (C.c_int, [VP, P(C.c_int), C.c_int, C.c_uint64, C.c_float, VP]),
}

# include/vrc_nn.h (learned upsampler kernels): all return int status
_I, _F, _LL = C.c_int, C.c_float, C.c_longlong
NN_SIGNATURES = {
    "vrc_nn_conv3x3_fwd": [VP, _I, _I, _I, _I, VP, VP, _I, _I, VP, _I, VP],
    "vrc_nn_conv3x3_fwd_upcat": [VP, _I, VP, _I, _I, _I, _I, VP, VP, _I, _I, VP, _I, VP],
    "vrc_nn_conv3x3_wgrad": [VP, VP, _I, _I, _I, _I, _I, VP, VP, VP],
    "vrc_nn_flip_weights": [VP, _I, _I, VP, VP],
    "vrc_nn_relu_bwd": [VP, VP, _LL, _I, VP],
    "vrc_nn_avgpool2": [VP, _I, _I, _I, _I, _F, VP, VP],
    "vrc_nn_upsample2": [VP, _I, _I, _I, _I, _F, VP, VP],
    "vrc_nn_concat": [VP, _I, VP, _I, _LL, VP, _I, VP],
    "vrc_nn_add": [VP, VP, _LL, VP],
    "vrc_nn_head_fwd": [VP, VP, _I, _I, _I, VP, VP],
    "vrc_nn_head_bwd": [VP, _I, _I, _I, VP, VP],
    "vrc_nn_bilinear_up2": [VP, _I, _I, _I, VP, VP],
    "vrc_nn_loss": [VP, VP, _I, _I, _I, _I, _F, VP, VP, VP, VP],
    "vrc_nn_adam": [VP, VP, VP, VP, VP, _LL, _F, _F, _F, _F, _I, VP],
    "vrc_nn_pack_input": [VP, VP, _LL, VP, VP],
    "vrc_nn_probe_error": [VP, VP, _I, _I, _I, _I, _I, VP, VP],
    "vrc_nn_tile_alpha": [VP, _I, _I, _I, _I, _I, VP, VP],
    "vrc_nn_conv3x3_tc": [VP, _I, VP, _I, _I, _I, _I, VP, VP, _I, _I, _I, VP, _I, VP, VP],
    "vrc_nn_weights_tc": [VP, _I, _I, _I, _I, VP, VP],
    "vrc_nn_set_wait_limit": [C.c_ulonglong],
}

# include/vrc_processor.h: the CudaRaycaster processor shim
_S = C.c_char_p
PROC_SIGNATURES = {
    "vrcp_create": (C.c_int, [C.c_int, P(VP)]),
    "vrcp_destroy": (C.c_int, [VP]),
    "vrcp_class_name": (_S, []),
    "vrcp_category": (_S, []),
    "vrcp_set_float": (C.c_int, [VP, _S, C.c_float]),
    "vrcp_get_float": (C.c_int, [VP, _S, P(C.c_float)]),
    "vrcp_set_int": (C.c_int, [VP, _S, C.c_int]),
    "vrcp_get_int": (C.c_int, [VP, _S, P(C.c_int)]),
    "vrcp_set_string": (C.c_int, [VP, _S, _S]),
    "vrcp_get_string": (C.c_int, [VP, _S, C.c_char_p, C.c_int]),
    "vrcp_set_floatv": (C.c_int, [VP, _S, P(C.c_float), C.c_int]),
    "vrcp_get_floatv": (C.c_int, [VP, _S, P(C.c_float), C.c_int]),
    "vrcp_set_intv": (C.c_int, [VP, _S, P(C.c_int), C.c_int]),
    "vrcp_get_intv": (C.c_int, [VP, _S, P(C.c_int), C.c_int]),
    "vrcp_set_camera": (C.c_int, [VP, P(Camera)]),
    "vrcp_get_camera": (C.c_int, [VP, P(Camera)]),
    "vrcp_set_tf_keys": (C.c_int, [VP, P(TFKey), C.c_int, C.c_float, C.c_float, C.c_float]),
    "vrcp_set_tf_domain": (C.c_int, [VP, C.c_float, C.c_float, C.c_int, C.c_int]),
    "vrcp_get_tf": (C.c_int, [VP, P(C.c_int), P(C.c_float), P(C.c_float), P(C.c_int)]),
    "vrcp_load_tf": (C.c_int, [VP, C.c_char_p]),
    "vrcp_set_volume": (C.c_int, [VP, P(VolumeDesc), VP]),
    "vrcp_set_entry_exit": (C.c_int, [VP, VP, VP, C.c_int, C.c_int]),
    "vrcp_set_output_size": (C.c_int, [VP, C.c_int, C.c_int]),
    "vrcp_is_ready": (C.c_int, [VP]),
    "vrcp_initialize": (None, [VP]),
    "vrcp_deinitialize": (None, [VP]),
    "vrcp_process": (None, [VP, C.c_int, C.c_int]),
    "vrcp_output": (C.c_int, [VP, P(P(C.c_float)), P(C.c_int), P(C.c_int)]),
    "vrcp_last_error": (_S, [VP]),
    "vrcp_last_stats": (C.c_int, [VP, P(RenderStats)]),
    "vrcp_invalidated": (C.c_int, [VP]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libvrc.so. Raises OSError/RuntimeError when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"voreen_gb300 CUDA library not built: {path} is missing (run __graft_entry__.build())")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    for name, args in NN_SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = C.c_int
        fn.argtypes = args
    for name, (res, args) in PROC_SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
