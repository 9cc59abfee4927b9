"""ctypes binding of the C ABI in include/isti.h (libisti.so).

The library is the product's only compute path.  Loading fails loudly when it
has not been built: there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

ISTI_OK = 0
ISTI_ERR_INVALID_ARG = 1
ISTI_ERR_OOM = 2
ISTI_ERR_CUDA = 3
ISTI_ERR_TIMEOUT = 4
ISTI_ERR_UNSUPPORTED = 5

ARITH_IEEE = 0           # ISTI_ARITH_IEEE
ARITH_REFERENCE_GPU = 1  # ISTI_ARITH_REFERENCE_GPU

MODE_OURS = 0
MODE_BACKWARD_BIDIRECTIONAL = 1
MODE_BACKWARD_UNIDIRECTIONAL = 2
MODE_SPLATTING = 3
MODE_TIMEWARP = 4

MOTION_NONE = 0
MOTION_F32X4 = 1
MOTION_F16X3 = 2

MAX_AUX_CAMS = 7

Mat16 = C.c_float * 16


class IstiView(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32),
        ("color", C.c_void_p), ("z", C.c_void_p), ("motion", C.c_void_p),
        ("motion_format", C.c_int32),
        ("shadow_color_a", C.c_void_p), ("shadow_color_b", C.c_void_p), ("shadow_info", C.c_void_p),
        ("viewproj", Mat16), ("inv_viewproj", Mat16),
    ]


class IstiFrameData(C.Structure):
    _fields_ = [
        ("fwd", IstiView), ("bwd", IstiView), ("num_aux", C.c_int32),
        ("aux_curr", C.POINTER(IstiView)), ("aux_next", C.POINTER(IstiView)),
        ("aux_priority", C.POINTER(C.c_int32)),
    ]


class IstiRenderInfo(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("alpha", C.c_float),
        ("viewproj", Mat16), ("inv_viewproj", Mat16),
        ("frames_per_anchor", C.c_int32), ("shadow_frames_per_anchor", C.c_int32),
        ("no_shadows", C.c_int32), ("mode", C.c_int32),
    ]


class IstiTiming(C.Structure):
    _fields_ = [("frames", C.c_int32), ("kernel_launches", C.c_int32), ("init_ms", C.c_float),
                ("splat_ms", C.c_float), ("reproj_ms", C.c_float)]


class IstiTuning(C.Structure):
    _fields_ = [("mode", C.c_int32), ("n_views", C.c_int32), ("n_frames", C.c_int32), ("shadows", C.c_int32),
                ("width", C.c_uint32), ("height", C.c_uint32), ("regs", C.c_int32), ("row_pairs", C.c_int32),
                ("best_ms", C.c_float), ("rule_ms", C.c_float), ("plain_tiles", C.c_int32)]


class IstiPairFrames(C.Structure):
    _fields_ = [("frame", C.POINTER(IstiFrameData)), ("n_frames", C.c_int32), ("out_rgba", C.POINTER(C.c_void_p)),
                ("infos", C.POINTER(IstiRenderInfo)), ("chain_outputs", C.c_int32)]


MAX_PAIRS = 64  # ISTI_MAX_PAIRS

# Every function include/isti.h declares: name -> (restype, argtypes)
SIGNATURES = {
    "isti_abi_version": (C.c_int32, []),
    "isti_last_error": (C.c_char_p, []),
    "isti_status_string": (C.c_char_p, [C.c_int]),
    "isti_renderer_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "isti_renderer_destroy": (C.c_int, [C.c_void_p]),
    "isti_render": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(IstiRenderInfo), C.POINTER(IstiFrameData), C.c_void_p]),
    "isti_renderer_view_buffers": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                             C.POINTER(C.c_void_p), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "isti_renderer_view_depth": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "isti_renderer_device_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "isti_renderer_set_pair_units": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "isti_renderer_test_stall_pair": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint32]),
    "isti_renderer_enable_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "isti_renderer_timing": (C.c_int, [C.c_void_p, C.POINTER(IstiTiming)]),
    "isti_renderer_set_autotune": (C.c_int, [C.c_void_p, C.c_int32]),
    "isti_renderer_set_reproj_launch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "isti_renderer_tuning_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "isti_renderer_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(IstiTuning)]),
    "isti_render_noalloc": (C.c_int, [C.c_void_p, C.POINTER(IstiRenderInfo), C.POINTER(IstiFrameData), C.c_void_p]),
    "isti_noalloc_device_status": (C.c_int, [C.POINTER(C.c_int32)]),
    "isti_renderer_set_arithmetic": (C.c_int, [C.c_void_p, C.c_int32]),
    "isti_renderer_test_withhold_tile": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_uint32]),
    "isti_render_batch": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(IstiRenderInfo),
                                    C.POINTER(IstiFrameData), C.c_int32, C.c_void_p]),
    "isti_render_pairs": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(IstiPairFrames), C.c_void_p]),
}


class IstiCameraInfo(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("client_fps", C.c_int32), ("server_fps", C.c_int32),
                ("shadow_fps", C.c_int32), ("priority", C.c_int32), ("n_frames", C.c_int32)]


class IstiCameraFrame(C.Structure):
    _fields_ = [("idx", C.c_int32), ("w2c", Mat16), ("proj", Mat16)]


_P = C.POINTER
_u8p, _f32p, _i32p = _P(C.c_uint8), _P(C.c_float), _P(C.c_int32)

# include/isti_io.h
IO_SIGNATURES = {
    "isti_png_decode_file": (C.c_int, [C.c_char_p, _i32p, _i32p, _P(_u8p)]),
    "isti_png_decode_memory": (C.c_int, [C.c_void_p, C.c_size_t, _i32p, _i32p, _P(_u8p)]),
    "isti_png_encode_file": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "isti_png_encode_memory": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, _P(_u8p), _P(C.c_size_t)]),
    "isti_exr_decode_file": (C.c_int, [C.c_char_p, _i32p, _i32p, _i32p, _P(_f32p)]),
    "isti_exr_decode_memory": (C.c_int, [C.c_void_p, C.c_size_t, _i32p, _i32p, _i32p, _P(_f32p)]),
    "isti_exr_encode_file": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32]),
    "isti_zlib_decompress": (C.c_int, [C.c_void_p, C.c_size_t, _P(_u8p), _P(C.c_size_t)]),
    "isti_image_free": (None, [C.c_void_p]),
}

# include/isti_dataset.h
DATASET_SIGNATURES = {
    "isti_camera_path_open": (C.c_int, [C.c_char_p, _P(C.c_void_p)]),
    "isti_camera_path_info": (C.c_int, [C.c_void_p, _P(IstiCameraInfo)]),
    "isti_camera_path_frame": (C.c_int, [C.c_void_p, C.c_int32, _P(IstiCameraFrame)]),
    "isti_camera_path_close": (None, [C.c_void_p]),
    "isti_dataset_open": (C.c_int, [C.c_char_p, C.c_int32, _P(C.c_char_p), C.c_void_p, _P(C.c_void_p)]),
    "isti_dataset_read_next": (C.c_int, [C.c_void_p, _i32p]),
    "isti_dataset_frame": (C.c_int, [C.c_void_p, _P(IstiFrameData)]),
    "isti_dataset_camera": (C.c_int, [C.c_void_p, C.c_int32, _P(IstiCameraInfo)]),
    "isti_dataset_matrices": (C.c_int, [C.c_void_p, C.c_int32, _f32p, _f32p]),
    "isti_dataset_keyframe": (C.c_int32, [C.c_void_p]),
    "isti_dataset_close": (None, [C.c_void_p]),
    "isti_depth_to_z": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "isti_normalize_proj": (C.c_int, [_f32p, _f32p]),
    "isti_rgb8_to_rgba8": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "isti_unpack_shadows": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
                                      C.c_void_p]),
    "isti_mat4_mul": (None, [_f32p, _f32p, _f32p]),
    "isti_mat4_inverse": (None, [_f32p, _f32p]),
    "isti_mat4_interpolate": (None, [_f32p, _f32p, C.c_float, _f32p]),
}

class IstiQuality(C.Structure):
    _fields_ = [("mse", C.c_double), ("psnr", C.c_double), ("ssim", C.c_double)]


# include/isti_metrics.h
METRICS_SIGNATURES = {
    "isti_quality_scratch_bytes": (C.c_size_t, [C.c_int32, C.c_int32]),
    "isti_quality_rgba8": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "isti_flip_scratch_bytes": (C.c_size_t, [C.c_int32, C.c_int32]),
    "isti_flip_rgba8": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p]),
}

FLIP_DEFAULT_PPD = 0.7 * 3840 / 0.7 * 3.141592653589793 / 180  # eval.py: 0.7 m wide 4K screen at 0.7 m

_VP = C.c_void_p
# include/isti_unet.h
UNET_SIGNATURES = {
    "isti_unet_packed_bytes": (C.c_size_t, [C.c_int32, C.c_int32, C.c_int32]),
    "isti_unet_pack": (C.c_int, [C.c_int32, _VP, C.c_int32, C.c_int32, C.c_int32, _VP, _VP]),
    "isti_unet_conv": (C.c_int, [C.c_int32, _VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _VP, _VP, _VP, C.c_int32, _VP, C.c_int32,
                                 _VP, _VP]),
    "isti_unet_wgrad_scratch_bytes": (C.c_size_t, [C.c_int32] * 6),
    "isti_unet_wgrad": (C.c_int, [C.c_int32, _VP, _VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _VP, C.c_int32, _VP,
                                  C.c_size_t, _VP, _VP]),
    "isti_flownet_input_channels": (C.c_int32, []),
    "isti_flownet_output_channels": (C.c_int32, []),
    "isti_flownet_num_layers": (C.c_int32, []),
    "isti_flownet_layer": (C.c_int, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
    "isti_flownet_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint64]),
    "isti_flownet_destroy": (C.c_int, [_VP]),
    "isti_flownet_tensors": (C.c_int, [_VP, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]),
    "isti_flownet_param_offsets": (C.c_int, [_VP, C.c_int32, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "isti_flownet_sync_params": (C.c_int, [_VP, _VP]),
    "isti_flownet_forward": (C.c_int, [_VP, _VP, C.c_int32, C.c_int32, C.c_int32, _VP, _VP, _VP]),
    "isti_flownet_backward": (C.c_int, [_VP, _VP, _VP, C.c_int32, C.c_int32, C.c_int32, _VP]),
    "isti_flownet_adam": (C.c_int, [_VP, C.c_float, _VP]),
    "isti_flownet_loss": (C.c_int, [_VP, C.POINTER(C.c_void_p)]),
    "isti_flownet_device_status": (C.c_int, [_VP, C.POINTER(C.c_int32)]),
    "isti_render_learned": (C.c_int, [_VP, _VP, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(IstiRenderInfo), C.POINTER(IstiFrameData),
                                      C.c_int32, C.c_int32, _VP]),
    "isti_renderer_learned_stats": (C.c_int, [_VP, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
}

# include/isti_train.h
TRAIN_SIGNATURES = {
    "isti_scene_raycast": (C.c_int, [_VP, C.c_int32, C.c_uint32, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double,
                                     C.c_double, _VP, _VP, _VP]),
    "isti_learned_grid": (C.c_int, [C.c_uint32, C.c_uint32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "isti_learned_input": (C.c_int, [_VP, C.c_int32, C.POINTER(IstiRenderInfo), C.POINTER(IstiFrameData), _VP, _VP]),
    "isti_learned_labels": (C.c_int, [_VP, C.c_int32, _VP, _VP]),
}

ALL_SIGNATURES = {**SIGNATURES, **IO_SIGNATURES, **DATASET_SIGNATURES, **METRICS_SIGNATURES, **UNET_SIGNATURES, **TRAIN_SIGNATURES}

MAX_BATCH_FRAMES = 8  # ISTI_MAX_BATCH_FRAMES

NOALLOC_SCRATCH_BYTES = 64 << 20  # ISTI_NOALLOC_SCRATCH_BYTES


class IstiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"isti status {status}: {msg}")
        self.status = status


_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load libisti.so (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or _build.cuda_lib_path()
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build the CUDA extension first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(p)
    for name, (res, args) in ALL_SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != ISTI_OK:
        lib = load()
        raise IstiError(status, lib.isti_last_error().decode(errors="replace"))


def mat16(m) -> Mat16:
    """Row-major 4x4 (numpy math convention) -> column-major float[16]."""
    import numpy as np
    a = np.asarray(m, dtype=np.float32).reshape(4, 4)
    return Mat16(*a.T.reshape(-1).tolist())
