"""ctypes front of the CPU oracle (test infrastructure only).

The oracle restates jixel 0.5.14's scalar UltraFast VarDCT front end in C
(``oracle/jxg_oracle.c``).  Tests, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` call it as the checker; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libjxg_oracle.so")

NUM_FINE_AC_CONTEXTS = 30 * (37 + 458)
ALPHABET = 128


class OrcParams(ctypes.Structure):
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
        ("x_qm_mul", ctypes.c_float),
        ("b_qm_mul", ctypes.c_float),
    ]


class OrcFrame(ctypes.Structure):
    _fields_ = [
        ("pixels", ctypes.c_void_p),
        ("bits", ctypes.c_int32),
        ("channels", ctypes.c_int32),
        ("transfer", ctypes.c_int32),
        ("speed", ctypes.c_int32),
        ("width", ctypes.c_uint64),
        ("height", ctypes.c_uint64),
        ("distance", ctypes.c_float),
        ("num_threads", ctypes.c_int32),
        ("xyb", ctypes.c_void_p),
        ("quant_field", ctypes.c_void_p),
        ("ytox", ctypes.c_void_p),
        ("ytob", ctypes.c_void_p),
        ("quant_dc", ctypes.c_void_p),
        ("coeffs", ctypes.c_void_p),
        ("nzeros", ctypes.c_void_p),
        ("tokens", ctypes.c_void_p),
        ("token_capacity", ctypes.c_uint64),
        ("group_offsets", ctypes.c_void_p),
        ("histograms", ctypes.c_void_p),
        ("alpha", ctypes.c_void_p),
        ("ac_strategy", ctypes.c_void_p),
        ("params", OrcParams),
        ("qf_threshold", ctypes.c_uint32),
        ("constant_blocks", ctypes.c_uint64),
        ("screen_content", ctypes.c_int32),
        ("epf_sharpness", ctypes.c_int32),
        ("num_tokens", ctypes.c_uint64),
        ("stage_seconds", ctypes.c_double * 5),
    ]


def build() -> None:
    """Compile the oracle with its Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_distance_from_quality.restype = ctypes.c_float
        _lib.orc_distance_from_quality.argtypes = [ctypes.c_float]
        _lib.orc_params_for.restype = ctypes.c_int
        _lib.orc_params_for.argtypes = [ctypes.c_float, ctypes.POINTER(OrcParams)]
        _lib.orc_dct8_tables.restype = ctypes.c_int
        _lib.orc_dct8_tables.argtypes = [ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
        _lib.orc_frontend.restype = ctypes.c_int
        _lib.orc_frontend.argtypes = [ctypes.POINTER(OrcFrame)]
        _lib.orc_sizeof_frame.restype = ctypes.c_uint64
        _lib.orc_epf_sharpness_id.restype = ctypes.c_int32
        _lib.orc_epf_sharpness_id.argtypes = [ctypes.c_float, ctypes.c_int]
        _lib.orc_fast_exp2.restype = ctypes.c_float
        _lib.orc_fast_exp2.argtypes = [ctypes.c_float]
        _lib.orc_dirty_log2f.restype = ctypes.c_float
        _lib.orc_dirty_log2f.argtypes = [ctypes.c_float]
        _lib.orc_hybrid_token.restype = ctypes.c_uint32
        _lib.orc_hybrid_token.argtypes = [ctypes.c_uint32]
        _lib.orc_freq_context.restype = ctypes.c_int32
        _lib.orc_freq_context.argtypes = [ctypes.c_int32]
        _lib.orc_nonzero_context.restype = ctypes.c_int32
        _lib.orc_nonzero_context.argtypes = [ctypes.c_int32]
        _lib.orc_chroma_hf_protection.restype = None
        _lib.orc_chroma_hf_protection.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                                  ctypes.c_float, ctypes.c_void_p]
        _lib.orc_pixel_chromacity.restype = None
        _lib.orc_pixel_chromacity.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                              ctypes.c_void_p, ctypes.c_void_p]
        _lib.orc_constant_blocks.restype = ctypes.c_uint64
        _lib.orc_constant_blocks.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]
        _lib.orc_strategy_cost_probe.restype = ctypes.c_float
        _lib.orc_strategy_cost_probe.argtypes = [
            ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_float, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_float]
        _lib.orc_fastest_select.restype = ctypes.c_int
        _lib.orc_fastest_select.argtypes = [
            ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint32, ctypes.c_void_p,
            ctypes.c_void_p]
        _lib.orc_large_tables.restype = ctypes.c_int
        _lib.orc_large_tables.argtypes = [ctypes.c_float] + [ctypes.c_void_p] * 4
        _lib.orc_natural_scan.restype = None
        _lib.orc_natural_scan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        assert _lib.orc_sizeof_frame() == ctypes.sizeof(OrcFrame), "OrcFrame layout mismatch"
    return _lib


def distance_from_quality(q: float) -> float:
    return float(lib().orc_distance_from_quality(q))


def params(distance: float) -> dict:
    p = OrcParams()
    st = lib().orc_params_for(distance, ctypes.byref(p))
    if st:
        raise ValueError(f"oracle params status {st}")
    return {
        "distance": p.distance,
        "global_scale": p.global_scale,
        "quant_dc": p.quant_dc,
        "scale": p.scale,
        "scale_dc": p.scale_dc,
        "x_qm_scale": p.x_qm_scale,
        "b_qm_scale": p.b_qm_scale,
        "epf_iters": p.epf_iters,
        "dc_step": list(p.dc_step),
        "x_qm_mul": p.x_qm_mul,
        "b_qm_mul": p.b_qm_mul,
    }


def dct8_tables(distance: float):
    m = np.zeros(192, np.float32)
    inv = np.zeros(192, np.float32)
    st = lib().orc_dct8_tables(distance, m.ctypes.data, inv.ctypes.data)
    if st:
        raise ValueError(f"oracle tables status {st}")
    return m.reshape(3, 64), inv.reshape(3, 64)


def natural_scan_8x8() -> np.ndarray:
    s = np.zeros(64, np.uint8)
    lib().orc_natural_scan_8x8(s.ctypes.data_as(ctypes.c_void_p))
    return s


def dct8x8(block: np.ndarray) -> np.ndarray:
    b = np.ascontiguousarray(block, np.float32).reshape(64)
    out = np.zeros(64, np.float32)
    lib().orc_dct8x8(b.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
    return out


@dataclass
class OracleFrame:
    width: int
    height: int
    params: dict
    xyb: np.ndarray
    quant_field: np.ndarray
    ytox: np.ndarray
    ytob: np.ndarray
    quant_dc: np.ndarray
    coeffs: np.ndarray
    nzeros: np.ndarray
    tokens: np.ndarray          # (N, 2) uint32: context, value
    group_offsets: np.ndarray
    histograms: np.ndarray      # (contexts, 128) uint32
    alpha: np.ndarray | None    # (h, w) uint16 alpha after fringe clearing (RGBA only)
    ac_strategy: np.ndarray
    qf_threshold: int
    constant_blocks: int
    screen_content: bool
    epf_sharpness: int
    stage_seconds: list


SPEEDS = {"ultrafast": 0, "fastest": 1}


def frontend(pixels: np.ndarray, distance: float, num_threads: int = 0,
             keep_coeffs: bool = True, bits: int | None = None,
             transfer: int = 0, speed: str = "ultrafast") -> OracleFrame:
    """Run the oracle on an (h, w, c) uint8 or uint16 image: `bits` 8, or
    10 / 12 / 16 for uint16 samples (default: the sample type's), `transfer`
    an H.273 transfer code (0: sRGB, the default encoding; 8: linear),
    `speed` "ultrafast" or "fastest"."""
    pixels = np.ascontiguousarray(pixels)
    if pixels.ndim == 2:  # grey
        pixels = pixels[:, :, None]
    h, w, ch = pixels.shape
    if bits is None:
        bits = 8 if pixels.dtype == np.uint8 else 16
    xb, yb = (w + 7) // 8, (h + 7) // 8
    tx, ty = (xb + 7) // 8, (yb + 7) // 8
    ng = ((w + 255) // 256) * ((h + 255) // 256)
    cap = xb * yb * 192
    xyb = np.zeros((3, h, w), np.float32)
    qf = np.zeros((yb, xb), np.uint8)
    ytox = np.zeros((ty, tx), np.int8)
    ytob = np.zeros((ty, tx), np.int8)
    qdc = np.zeros((3, yb, xb), np.int16)
    coeffs = np.zeros((yb, xb, 3, 64), np.int32) if keep_coeffs else None
    nz = np.zeros((3, yb, xb), np.uint8)
    tokens = np.zeros((cap, 2), np.uint32)
    offs = np.zeros(ng + 1, np.uint64)
    hist = np.zeros((NUM_FINE_AC_CONTEXTS, ALPHABET), np.uint32)
    alpha = np.zeros((h, w), np.uint16) if ch in (2, 4) else None
    strategy = np.zeros((yb, xb), np.uint8)
    f = OrcFrame()
    f.speed = SPEEDS[speed]
    f.pixels = pixels.ctypes.data
    f.bits = bits
    f.transfer = transfer
    f.channels = ch
    f.width = w
    f.height = h
    f.distance = distance
    f.num_threads = num_threads
    f.xyb = xyb.ctypes.data
    f.quant_field = qf.ctypes.data
    f.ytox = ytox.ctypes.data
    f.ytob = ytob.ctypes.data
    f.quant_dc = qdc.ctypes.data
    f.coeffs = coeffs.ctypes.data if coeffs is not None else None
    f.nzeros = nz.ctypes.data
    f.tokens = tokens.ctypes.data
    f.token_capacity = cap
    f.group_offsets = offs.ctypes.data
    f.histograms = hist.ctypes.data
    f.alpha = alpha.ctypes.data if alpha is not None else None
    f.ac_strategy = strategy.ctypes.data
    st = lib().orc_frontend(ctypes.byref(f))
    if st:
        raise ValueError(f"oracle frontend status {st}")
    p = f.params
    return OracleFrame(
        width=w, height=h,
        params={"distance": p.distance, "global_scale": p.global_scale, "quant_dc": p.quant_dc,
                "scale": p.scale, "scale_dc": p.scale_dc, "x_qm_scale": p.x_qm_scale,
                "b_qm_scale": p.b_qm_scale, "epf_iters": p.epf_iters,
                "dc_step": list(p.dc_step)},
        xyb=xyb, quant_field=qf, ytox=ytox, ytob=ytob, quant_dc=qdc, coeffs=coeffs,
        nzeros=nz, tokens=tokens[: f.num_tokens], group_offsets=offs, histograms=hist, alpha=alpha,
        ac_strategy=strategy,
        qf_threshold=f.qf_threshold, constant_blocks=f.constant_blocks,
        screen_content=bool(f.screen_content), epf_sharpness=f.epf_sharpness,
        stage_seconds=list(f.stage_seconds),
    )


def alpha_fringe_clear(alpha: np.ndarray, maxv: int) -> np.ndarray:
    """alpha_fringe::clear on a copy of an (h, w) integer alpha plane."""
    a = np.ascontiguousarray(alpha, np.uint16).copy()
    h, w = a.shape
    lib().orc_alpha_fringe_clear(a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(w),
                                 ctypes.c_size_t(h), ctypes.c_uint32(maxv))
    return a


def fill_invisible(xyb: np.ndarray, alpha: np.ndarray) -> np.ndarray:
    """invisible::fill_invisible on a copy of (3, h, w) float planes."""
    x = np.ascontiguousarray(xyb, np.float32).copy()
    a = np.ascontiguousarray(alpha, np.uint16)
    _, h, w = x.shape
    lib().orc_fill_invisible(x.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                             ctypes.c_size_t(w), ctypes.c_size_t(h))
    return x


def alpha_block_factors(alpha: np.ndarray, maxv: int) -> np.ndarray:
    """alpha_block_factors of an (h, w) integer alpha plane: (yb, xb) float32."""
    a = np.ascontiguousarray(alpha, np.uint16)
    h, w = a.shape
    out = np.zeros(((h + 7) // 8, (w + 7) // 8), np.float32)
    lib().orc_alpha_block_factors(a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(w),
                                  ctypes.c_size_t(h), ctypes.c_uint32(maxv),
                                  out.ctypes.data_as(ctypes.c_void_p))
    return out


def dct8_default_bands() -> np.ndarray:
    out = np.zeros(18, np.float32)
    lib().orc_dct8_default_bands(out.ctypes.data_as(ctypes.c_void_p))
    return out.reshape(3, 6)


def dct8_matrix_from_bands(bands: np.ndarray) -> np.ndarray:
    """compute_dct8x8_matrix of (3, 6) band parameters: (3, 64) weights."""
    b = np.ascontiguousarray(bands, np.float32).reshape(18)
    m = np.zeros(192, np.float32)
    inv = np.zeros(192, np.float32)
    lib().orc_dct8_matrix_from_bands(b.ctypes.data_as(ctypes.c_void_p),
                                     m.ctypes.data_as(ctypes.c_void_p),
                                     inv.ctypes.data_as(ctypes.c_void_p))
    return m.reshape(3, 64)


def cmap_tile0(xyb: np.ndarray, distance: float) -> tuple[int, int]:
    """compute_cmap_tile of the first 64x64 tile of (3, h, w) XYB planes."""
    x = np.ascontiguousarray(xyb, np.float32)
    _, h, w = x.shape
    ytox, ytob = ctypes.c_int8(), ctypes.c_int8()
    st = lib().orc_cmap_tile0(x.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(w),
                              ctypes.c_size_t(h), ctypes.c_float(distance), ctypes.byref(ytox),
                              ctypes.byref(ytob))
    assert st == 0
    return ytox.value, ytob.value


def srgb_lut() -> np.ndarray:
    out = np.zeros(256, np.float32)
    lib().orc_srgb_lut(out.ctypes.data_as(ctypes.c_void_p))
    return out


# AcToken storage (src/entropy/token_stream.rs:32-48): 14 context bits over
# 18 value bits in one u32.
PACKED_VALUE_BITS = 18
PACKED_MAX_VALUE = (1 << PACKED_VALUE_BITS) - 1
PACKED_MAX_CONTEXT = (1 << (32 - PACKED_VALUE_BITS)) - 1


def ac_tokens_from(tokens: np.ndarray, group_offsets: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """`AcTokens::from` (src/entropy/token_stream.rs:59-76) applied to each
    group's tokens, as `process_ac_group` stores them
    (src/frame/ac_groups.rs:243): a group whose OR of contexts is at most
    PACKED_MAX_CONTEXT and OR of values at most PACKED_MAX_VALUE becomes one
    word per token (context << 18 | value); any other group keeps its
    (context, value) pairs.  Returns the concatenated words and the groups'
    word offsets (from zero)."""
    tokens = np.asarray(tokens, np.uint32).reshape(-1, 2)
    goffs = np.asarray(group_offsets, np.uint64)
    base = int(goffs[0])
    parts, woffs = [], [0]
    for g in range(len(goffs) - 1):
        t = tokens[int(goffs[g]) - base:int(goffs[g + 1]) - base]
        ctx_or = int(np.bitwise_or.reduce(t[:, 0])) if len(t) else 0
        val_or = int(np.bitwise_or.reduce(t[:, 1])) if len(t) else 0
        if ctx_or <= PACKED_MAX_CONTEXT and val_or <= PACKED_MAX_VALUE:
            parts.append((t[:, 0] << np.uint32(PACKED_VALUE_BITS)) | t[:, 1])
        else:
            parts.append(t.reshape(-1))
        woffs.append(woffs[-1] + len(parts[-1]))
    words = np.concatenate(parts).astype(np.uint32) if parts else np.zeros(0, np.uint32)
    return words, np.asarray(woffs, np.uint64)


def ac_token_unpack(word: int) -> tuple[int, int]:
    """`AcToken::unpack` (src/entropy/token_stream.rs:44-48)."""
    return word >> PACKED_VALUE_BITS, word & PACKED_MAX_VALUE


# DctFn kinds of orc_dct: name (rows x columns) -> (kind, W, H, DC values)
DCT_KINDS = {
    "8x8": (0, 8, 8, 1), "8x16": (1, 16, 8, 2), "16x8": (2, 8, 16, 2), "16x16": (3, 16, 16, 4),
    "16x32": (4, 32, 16, 8), "32x16": (5, 16, 32, 8), "32x32": (6, 32, 32, 16),
    "32x8": (7, 8, 32, 4), "8x32": (8, 32, 8, 4), "64x64": (9, 64, 64, 64),
    "64x32": (10, 32, 64, 32), "32x64": (11, 64, 32, 32),
    "128x128": (12, 128, 128, 256), "128x64": (13, 64, 128, 128), "64x128": (14, 128, 64, 128),
}


def dct(name: str, block: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """`DctFn<W, H, N>` of one (H, W) block (src/dct.rs: dct8x16 :823, dct16x8
    :904, dct16x16 :1010, dct32x32 :1980, dct32x16 :2251, dct16x32 :2340,
    dct32x8 :1742, dct8x32 :1777, dct64x64 :2576, dct64x32 :2659, dct32x64
    :2689; src/dct128.rs dct128x128 :385, dct128x64 :416, dct64x128 :446) and
    its per-8x8 DC values (dc_from_dct*): (N coefficients, DC values)."""
    kind, w, h, ndc = DCT_KINDS[name]
    b = np.ascontiguousarray(block, np.float32).reshape(h, w)
    out = np.zeros(w * h, np.float32)
    dc = np.zeros(ndc, np.float32)
    assert lib().orc_dct(ctypes.c_int(kind), b.ctypes.data_as(ctypes.c_void_p),
                         out.ctypes.data_as(ctypes.c_void_p), dc.ctypes.data_as(ctypes.c_void_p)) == 0
    return out, dc


def dct1d(vec: np.ndarray) -> np.ndarray:
    """dct1d_8 / dct1d_16 / dct1d_32 / dct1d_64 (src/dct.rs:109, :687, :1477,
    :2529) / dct1d_128 (src/dct128.rs:330) of one vector."""
    v = np.ascontiguousarray(vec, np.float32).copy()
    assert v.size in (8, 16, 32, 64, 128)
    lib().orc_dct1d(v.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(v.size))
    return v


def gaborish_inverse(xyb: np.ndarray, mul: float = 0.9908511) -> np.ndarray:
    """gaborish_inverse (src/gaborish.rs:44) of (3, h, w) planes: a new array."""
    x = np.ascontiguousarray(xyb, np.float32)
    out = np.zeros_like(x)
    lib().orc_gaborish_inverse(x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
                               ctypes.c_size_t(x.shape[2]), ctypes.c_size_t(x.shape[1]),
                               ctypes.c_float(mul))
    return out


def gaborish_inverse_weights(mul: float = 0.9908511) -> np.ndarray:
    w = np.zeros(6, np.float32)
    lib().orc_gaborish_inverse_weights(ctypes.c_float(mul), w.ctypes.data_as(ctypes.c_void_p))
    return w


def gaborish(xyb: np.ndarray) -> np.ndarray:
    """The decoder's Gaborish (src/epf_filter.rs:165) of (3, h, w) planes."""
    x = np.ascontiguousarray(xyb, np.float32)
    out = np.zeros_like(x)
    lib().orc_gaborish(x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
                       ctypes.c_size_t(x.shape[2]), ctypes.c_size_t(x.shape[1]))
    return out


def gaborish_weights() -> np.ndarray:
    w = np.zeros(3, np.float32)
    lib().orc_gaborish_weights(w.ctypes.data_as(ctypes.c_void_p))
    return w


def idct(name: str, coeffs: np.ndarray) -> np.ndarray:
    """The inverse of `dct(name, ...)` (IdctMethods, src/dct.rs:358-416;
    inv_dct8x16 :1634, inv_dct16x8 :1658, inv_dct16x32 :1683, inv_dct32x16
    :1705, the square inverses :1590-1620): (H, W) samples."""
    kind, w, h, _ = DCT_KINDS[name]
    c = np.ascontiguousarray(coeffs, np.float32).reshape(-1)
    assert c.size == w * h
    out = np.zeros((h, w), np.float32)
    assert lib().orc_idct(ctypes.c_int(kind), c.ctypes.data_as(ctypes.c_void_p),
                          out.ctypes.data_as(ctypes.c_void_p)) == 0
    return out


# The 8x8-sized transforms besides DCT8 (orc_small_transform kinds)
SMALL_TRANSFORMS = {"identity": 0, "dct2x2": 1, "dct4x4": 2, "dct4x8": 3, "dct8x4": 4,
                    "inv_identity": 5, "inv_dct2x2": 6,
                    "afv0": 7, "afv1": 8, "afv2": 9, "afv3": 10}


def small_transform(name: str, block: np.ndarray) -> np.ndarray:
    """identity8x8 (src/dct.rs:185), dct2x2_8x8 (:306), dct4x4 (:1163),
    dct4x8 (:1238), dct8x4 (:1319), inv_identity8x8 (:225), inv_dct2x2_8x8
    (:345), afv_from_pixels (src/afv.rs:207, afv0..afv3) of one 8x8 block:
    64 values."""
    b = np.ascontiguousarray(block, np.float32).reshape(64)
    out = np.zeros(64, np.float32)
    assert lib().orc_small_transform(ctypes.c_int(SMALL_TRANSFORMS[name]),
                                     b.ctypes.data_as(ctypes.c_void_p),
                                     out.ctypes.data_as(ctypes.c_void_p)) == 0
    return out


def afv_basis() -> np.ndarray:
    """The oracle's AFV basis (src/afv.rs:48-180) as [vector][pixel], 16x16."""
    out = np.zeros(256, np.float32)
    lib().orc_afv_basis(out.ctypes.data_as(ctypes.c_void_p))
    return out.reshape(16, 16)


def dct4_2d(block: np.ndarray) -> np.ndarray:
    """dct4x4_2d (src/dct.rs:1061) of a 4x4 block (16 values, transposed
    output) or dct4x8_2d (:1198) of a 4-row, 8-column block (32 values)."""
    b = np.ascontiguousarray(block, np.float32).reshape(-1).copy()
    out = np.zeros_like(b)
    fn = {16: lib().orc_dct4x4_2d, 32: lib().orc_dct4x8_2d}[b.size]
    fn(b.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
    return out


def transfer_lut(bits: int, transfer: int) -> np.ndarray:
    """TransferLut::build (src/color.rs:297-333): 256 entries for 8-bit
    samples, 65536 otherwise."""
    out = np.zeros(65536, np.float32)
    st = lib().orc_transfer_lut(ctypes.c_int(bits), ctypes.c_int(transfer),
                                out.ctypes.data_as(ctypes.c_void_p))
    if st:
        raise ValueError(f"transfer {transfer} at {bits} bits: status {st}")
    return out[:256] if bits == 8 else out


def chroma_hf_protection(xyb: np.ndarray, distance: float, field: np.ndarray) -> np.ndarray:
    """apply_chroma_hf_protection (src/adaptive_quant.rs:303-402) of (3, h, w)
    XYB planes on a copy of the (yb, xb) u8 field."""
    xyb = np.ascontiguousarray(xyb, np.float32)
    _, h, w = xyb.shape
    out = np.ascontiguousarray(field, np.uint8).copy()
    lib().orc_chroma_hf_protection(xyb.ctypes.data, w, h, float(distance), out.ctypes.data)
    return out


def pixel_chromacity(xyb: np.ndarray) -> tuple[np.ndarray, int, int]:
    """pixel_chromacity_steps (src/frame/chroma.rs:89-165) of (3, h, w) XYB
    planes: the seven counts (X steps at three levels, B - Y steps at three,
    exposed blue) and the extra X and B quant-scale steps."""
    xyb = np.ascontiguousarray(xyb, np.float32)
    _, h, w = xyb.shape
    counts = np.zeros(7, np.uint32)
    steps = np.zeros(2, np.uint32)
    lib().orc_pixel_chromacity(xyb.ctypes.data, w, h, counts.ctypes.data, steps.ctypes.data)
    return counts, int(steps[0]), int(steps[1])


def natural_scan(cx: int, cy: int) -> np.ndarray:
    """natural_scan_generic: scan position -> raw index of a cx >= cy block."""
    out = np.zeros(cx * cy * 64, np.uint16)
    lib().orc_natural_scan(cx, cy, out.ctypes.data)
    return out


def strategy_cost(xyb: np.ndarray, ytox: np.ndarray, ytob: np.ndarray, distance: float,
                  strategy: int, bx: int, by: int, qac: float) -> float:
    """strategy_cost (coefficient model, META_R) of one candidate transform
    with its first block at (bx, by), on (3, h, w) XYB planes and the frame's
    CfL tile maps."""
    x = np.ascontiguousarray(xyb, np.float32)
    tx = np.ascontiguousarray(ytox, np.int8)
    tb = np.ascontiguousarray(ytob, np.int8)
    _, h, w = x.shape
    return float(lib().orc_strategy_cost_probe(x.ctypes.data, w, h, tx.ctypes.data, tb.ctypes.data,
                                               distance, strategy, bx, by, qac))


def fastest_select(xyb: np.ndarray, ytox: np.ndarray, ytob: np.ndarray, qf: np.ndarray,
                   ctx_distance: float, distance: float, scale: float,
                   x_qm_scale: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """fill_ac_strategy at Fastest on one (3, h, w) image: returns the
    strategy map (raw << 1 | first per block) and the adjusted quant field."""
    x = np.ascontiguousarray(xyb, np.float32)
    _, h, w = x.shape
    q = np.ascontiguousarray(qf, np.uint8).copy()
    m = np.zeros_like(q)
    tx = np.ascontiguousarray(ytox, np.int8)
    tb = np.ascontiguousarray(ytob, np.int8)
    st = lib().orc_fastest_select(x.ctypes.data, w, h, tx.ctypes.data, tb.ctypes.data,
                                  ctx_distance, distance, scale, x_qm_scale, q.ctypes.data,
                                  m.ctypes.data)
    if st:
        raise ValueError(f"oracle fastest_select status {st}")
    return m, q


def large_tables(distance: float) -> dict:
    """DequantMatrices::new_fast's 16x8, 16x16 and 32x32 forward matrices at
    `distance`, plus the 16x8 table recomputed from its band parameters."""
    out = {"16x8": np.zeros((3, 128), np.float32), "16x16": np.zeros((3, 256), np.float32),
           "32x32": np.zeros((3, 1024), np.float32), "16x8_bands": np.zeros((3, 128), np.float32)}
    st = lib().orc_large_tables(distance, out["16x8"].ctypes.data, out["16x16"].ctypes.data,
                                out["32x32"].ctypes.data, out["16x8_bands"].ctypes.data)
    if st:
        raise ValueError(f"oracle large_tables status {st}")
    return out
