"""ctypes binding of the C ABI declared in include/jxg.h.

The shared library is the product; it must be built (``jixel_gb300.build``)
before use.  There is no fallback path: a missing library raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libjxg.so")

# Every symbol include/jxg.h declares, in header order.
EXPORTS = [
    "jxg_context_create",
    "jxg_context_destroy",
    "jxg_context_set_stream",
    "jxg_context_last_error",
    "jxg_distance_from_quality",
    "jxg_frame_info_for",
    "jxg_validate_input",
    "jxg_frontend_run",
    "jxg_frontend_run_device",
    "jxg_frontend_params",
    "jxg_frontend_fetch",
    "jxg_frontend",
    "jxg_order_stats",
    "jxg_pixel_chromacity",
    "jxg_derive_orders",
    "jxg_frontend_enqueue",
    "jxg_frontend_wait",
    "jxg_batch_create",
    "jxg_batch_add",
    "jxg_batch_run",
    "jxg_batch_result",
    "jxg_batch_destroy",
    "jxg_op_fill_quant_field",
    "jxg_op_chroma_hf_protection",
    "jxg_op_gaborish_inverse",
    "jxg_op_gaborish",
    "jxg_op_epf",
    "jxg_op_luma_proxy",
    "jxg_op_epf_fit",
    "jxg_op_dct8x8",
    "jxg_op_pack_tokens",
    "jxg_op_dct",
    "jxg_op_idct",
    "jxg_op_small_transform",
    "jxg_token_offsets_noalloc",
    "jxg_selftest_bounded_wait",
    "jxg_selftest_token_lookback",
    "jxg_selftest_math",
    "jxg_refine_begin",
    "jxg_refine_eval",
    "jxg_refine_set_weights",
    "jxg_refine_step",
    "jxg_refine_theta",
    "jxg_refine_decoded",
    "jxg_refine_field",
    "jxg_refine_model",
    "jxg_frontend_run_with_field",
    "jxg_get_launch_geometry",
    "jxg_set_launch_geometry",
    "jxg_autotune",
    "jxg_enable_kernel_timing",
    "jxg_kernel_times",
    "jxg_reset_kernel_times",
]

NUM_FINE_AC_CONTEXTS = 14850
NOALLOC_MAX_GROUPS = 10922
TUNE_KERNELS = 10
ALPHABET_SIZE = 128


class Config(ctypes.Structure):
    _fields_ = [
        ("distance", ctypes.c_float),
        ("speed", ctypes.c_int32),
        ("num_threads", ctypes.c_int32),
        ("transfer", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 4),
    ]


class FrameInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "width", "height", "xsize_blocks", "ysize_blocks", "xsize_tiles", "ysize_tiles",
        "xsize_groups", "ysize_groups", "num_groups", "num_dc_groups", "max_tokens")]


class FrameParams(ctypes.Structure):
    _fields_ = [
        ("distance", ctypes.c_float),
        ("global_scale", ctypes.c_int32),
        ("quant_dc", ctypes.c_int32),
        ("scale", ctypes.c_float),
        ("scale_dc", ctypes.c_float),
        ("x_qm_scale", ctypes.c_uint32),
        ("b_qm_scale", ctypes.c_uint32),
        ("epf_iters", ctypes.c_uint32),
        ("dc_step", ctypes.c_float * 3),
        ("qf_threshold", ctypes.c_uint32),
        ("screen_content", ctypes.c_uint32),
        ("epf_sharpness", ctypes.c_int32),
        ("reserved", ctypes.c_uint32),
        ("constant_blocks", ctypes.c_uint64),
        ("num_tokens", ctypes.c_uint64),
    ]


class FrontendOutput(ctypes.Structure):
    _fields_ = [
        ("quant_field", ctypes.c_void_p),
        ("ac_strategy", ctypes.c_void_p),
        ("ytox_map", ctypes.c_void_p),
        ("ytob_map", ctypes.c_void_p),
        ("quant_dc", ctypes.c_void_p),
        ("coefficients", ctypes.c_void_p),
        ("num_nzeros", ctypes.c_void_p),
        ("xyb", ctypes.c_void_p),
        ("tokens", ctypes.c_void_p),
        ("token_capacity", ctypes.c_uint64),
        ("group_offsets", ctypes.c_void_p),
        ("histograms", ctypes.c_void_p),
        ("alpha", ctypes.c_void_p),
        ("packed_tokens", ctypes.c_void_p),
        ("packed_capacity", ctypes.c_uint64),
        ("packed_offsets", ctypes.c_void_p),
    ]


_lib = None


def load() -> ctypes.CDLL:
    """Load the in-tree library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m jixel_gb300.build` "
            "(the front end has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    vp, u64, i32, f32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_float
    sig = {
        "jxg_context_create": (i32, [i32, ctypes.POINTER(vp)]),
        "jxg_context_destroy": (None, [vp]),
        "jxg_context_set_stream": (i32, [vp, vp]),
        "jxg_context_last_error": (ctypes.c_char_p, [vp]),
        "jxg_distance_from_quality": (f32, [f32]),
        "jxg_frame_info_for": (i32, [u64, u64, ctypes.POINTER(FrameInfo)]),
        "jxg_validate_input": (i32, [u64, u64, i32, i32, ctypes.POINTER(Config)]),
        "jxg_frontend_run": (i32, [vp, vp, u64, u64, i32, i32, ctypes.POINTER(Config)]),
        "jxg_frontend_run_device": (i32, [vp, vp, u64, u64, i32, i32, ctypes.POINTER(Config)]),
        "jxg_frontend_params": (i32, [vp, ctypes.POINTER(FrameParams)]),
        "jxg_frontend_fetch": (i32, [vp, ctypes.POINTER(FrontendOutput)]),
        "jxg_frontend": (i32, [vp, vp, u64, u64, i32, i32, ctypes.POINTER(Config),
                               ctypes.POINTER(FrameParams), ctypes.POINTER(FrontendOutput)]),
        "jxg_order_stats": (i32, [vp, vp, vp]),
        "jxg_pixel_chromacity": (i32, [vp, vp, vp, vp]),
        "jxg_derive_orders": (i32, [vp, vp, vp, vp, vp]),
        "jxg_frontend_enqueue": (i32, [vp, vp, u64, u64, i32, i32, ctypes.POINTER(Config),
                                       ctypes.POINTER(FrameParams),
                                       ctypes.POINTER(FrontendOutput)]),
        "jxg_frontend_wait": (i32, [vp]),
        "jxg_batch_create": (i32, [vp, i32, ctypes.POINTER(vp)]),
        "jxg_batch_add": (ctypes.c_int64, [vp, vp, u64, u64, i32, i32, ctypes.POINTER(Config)]),
        "jxg_batch_run": (i32, [vp, i32]),
        "jxg_batch_result": (i32, [vp, u64, ctypes.POINTER(FrameParams),
                                   ctypes.POINTER(FrontendOutput)]),
        "jxg_batch_destroy": (None, [vp]),
        "jxg_op_fill_quant_field": (i32, [vp, vp, u64, u64, f32, f32, vp]),
        "jxg_op_chroma_hf_protection": (i32, [vp, vp, u64, u64, ctypes.c_float, vp]),
        "jxg_op_gaborish_inverse": (i32, [vp, vp, u64, u64, ctypes.c_float, vp]),
        "jxg_op_gaborish": (i32, [vp, vp, u64, u64, vp]),
        "jxg_op_epf": (i32, [vp, vp, u64, u64, vp, i32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, vp, i32, vp]),
        "jxg_op_luma_proxy": (i32, [vp, vp, vp, u64, u64, vp, vp]),
        "jxg_op_epf_fit": (i32, [vp, vp, vp, u64, u64, vp, ctypes.c_float, vp, vp]),
        "jxg_op_dct8x8": (i32, [vp, vp, u64, vp]),
        "jxg_op_pack_tokens": (i32, [vp, vp, vp, u64, vp, u64, vp]),
        "jxg_op_dct": (i32, [vp, i32, vp, u64, vp, vp]),
        "jxg_op_idct": (i32, [vp, i32, vp, u64, vp]),
        "jxg_op_small_transform": (i32, [vp, i32, vp, u64, vp]),
        "jxg_token_offsets_noalloc": (i32, [vp, u64, vp, vp, vp]),
        "jxg_selftest_bounded_wait": (i32, [vp, ctypes.c_uint32]),
        "jxg_selftest_token_lookback": (i32, [vp, ctypes.c_uint32]),
        "jxg_selftest_math": (i32, [vp, i32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(u64),
                                    ctypes.POINTER(ctypes.c_uint32)]),
        "jxg_refine_begin": (i32, [vp, vp, vp]),
        "jxg_refine_eval": (i32, [vp, vp, ctypes.c_float, vp, vp, vp]),
        "jxg_refine_set_weights": (i32, [vp, ctypes.c_float, ctypes.c_float]),
        "jxg_refine_step": (i32, [vp, ctypes.c_float, ctypes.c_float, vp]),
        "jxg_refine_theta": (i32, [vp, vp, i32]),
        "jxg_refine_decoded": (i32, [vp, vp, vp]),
        "jxg_refine_field": (i32, [vp, vp, vp]),
        "jxg_refine_model": (i32, [vp, vp, vp, vp, vp]),
        "jxg_frontend_run_with_field": (i32, [vp, vp, u64, u64, i32, i32, ctypes.POINTER(Config), vp, i32]),
        "jxg_get_launch_geometry": (i32, [vp, vp]),
        "jxg_set_launch_geometry": (i32, [vp, vp]),
        "jxg_autotune": (i32, [vp, vp, u64, u64, i32, i32, ctypes.POINTER(Config), i32, vp]),
        "jxg_enable_kernel_timing": (i32, [vp, i32]),
        "jxg_kernel_times": (i32, [vp, ctypes.POINTER(ctypes.c_char_p),
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(u64), i32]),
        "jxg_reset_kernel_times": (i32, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
