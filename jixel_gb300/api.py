"""Host-side mirror of the reference encoder's front-end interface.

Names follow jixel's public API (`EncodeConfig`, `Speed`, `EncodeError`,
`distance_from_quality`, src/encode_image.rs) and its stage boundary
(`DcGroupData` maps and `PendingAcGroup` tokens, src/dc_group_data.rs:325,
src/frame/ac_groups.rs:78).  Every call goes to the CUDA library through the
C ABI; nothing here computes a result itself.
"""
from __future__ import annotations

import ctypes
import enum
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


class Speed(enum.IntEnum):
    """`Speed` (src/encode_image.rs:256-286)."""
    ULTRA_FAST = 0
    FASTEST = 1
    FAST = 2
    MEDIUM = 3
    MEDIUM_SLOW = 4
    SLOW = 5
    EXTRA_SLOW = 6


class TransferFunction(enum.IntEnum):
    """`TransferFunction` (src/color_encoding.rs:99-160): H.273 codes."""
    BT709 = 1
    UNSPECIFIED = 2
    BT470M = 4
    BT470BG = 5
    BT601 = 6
    SMPTE240 = 7
    LINEAR = 8
    LOG100 = 9
    LOG100_SQRT10 = 10
    IEC61966 = 11
    BT1361 = 12
    SRGB = 13
    BT2020_10BIT = 14
    BT2020_12BIT = 15
    SMPTE2084 = 16
    SMPTE428 = 17
    HLG = 18


_ERRORS = {
    1: "EmptyImage", 2: "InputSizeMismatch", 3: "AlphaSizeMismatch", 4: "InvalidDistance",
    5: "QualityIsNaN", 6: "DimensionTooLarge", 7: "AllocationFailed", 8: "Unsupported",
    9: "BadChannelCount", 10: "BadBitDepth", 100: "InvalidArgument", 101: "Cuda",
    102: "DeviceTimeout",
}


class EncodeError(Exception):
    """`EncodeError` (src/util.rs:129-160); `variant` names the reference case."""

    def __init__(self, code: int, detail: str = ""):
        self.code = code
        self.variant = _ERRORS.get(code, f"Status{code}")
        super().__init__(f"{self.variant}: {detail}" if detail else self.variant)


def distance_from_quality(quality: float) -> float:
    """`distance_from_quality` (src/encode_image.rs:1321-1338)."""
    if quality != quality:
        raise EncodeError(5, "quality must not be NaN")
    return float(L.load().jxg_distance_from_quality(float(quality)))


@dataclass
class EncodeConfig:
    """The part of `EncodeConfig` (src/encode_image.rs:326-588) the front end
    reads.  `transfer` is `color_encoding.transfer` (default sRGB);
    `bits_per_sample` picks the entry point for uint16 samples, as
    encode_image_10bit / _12bit / _16bit do (0: 8 for uint8, 16 for uint16).
    The reference defaults to Speed.FAST; this build runs the UltraFast gates
    and, above distance 1.709, the Fastest ones, so its default is ULTRA_FAST
    (any other tier returns EncodeError Unsupported with the reason)."""
    distance: float = 1.0
    speed: Speed = Speed.ULTRA_FAST
    num_threads: int = field(default_factory=lambda: os.cpu_count() or 1)
    transfer: TransferFunction = TransferFunction.SRGB
    bits_per_sample: int = 0

    def with_transfer(self, transfer: TransferFunction) -> "EncodeConfig":
        self.transfer = TransferFunction(transfer)
        return self

    def with_bits_per_sample(self, bits: int) -> "EncodeConfig":
        self.bits_per_sample = int(bits)
        return self

    def with_quality(self, quality: float) -> "EncodeConfig":
        self.distance = distance_from_quality(quality)
        return self

    def with_distance(self, distance: float) -> "EncodeConfig":
        self.distance = float(distance)
        return self

    def with_speed(self, speed: Speed) -> "EncodeConfig":
        self.speed = Speed(speed)
        return self

    def with_num_threads(self, n: int) -> "EncodeConfig":
        self.num_threads = max(1, int(n))
        return self

    def _c(self) -> L.Config:
        c = L.Config()
        c.distance = self.distance
        c.speed = int(self.speed)
        c.num_threads = self.num_threads
        c.transfer = int(self.transfer)
        return c


def validate_input(width: int, height: int, channels: int, bits: int,
                   config: EncodeConfig) -> None:
    """Raise the `EncodeError` the front end would return for these inputs."""
    cfg = config._c()
    st = L.load().jxg_validate_input(width, height, channels, bits, ctypes.byref(cfg))
    if st:
        raise EncodeError(st)


@dataclass
class FrameInfo:
    width: int
    height: int
    xsize_blocks: int
    ysize_blocks: int
    xsize_tiles: int
    ysize_tiles: int
    xsize_groups: int
    ysize_groups: int
    num_groups: int
    num_dc_groups: int
    max_tokens: int


def frame_info(width: int, height: int) -> FrameInfo:
    fi = L.FrameInfo()
    st = L.load().jxg_frame_info_for(width, height, ctypes.byref(fi))
    if st:
        raise EncodeError(st)
    return FrameInfo(*[getattr(fi, n) for n, _ in L.FrameInfo._fields_])


@dataclass
class FrontendResult:
    """Pass-one output of the VarDCT front end for one frame."""
    params: dict
    quant_field: np.ndarray   # (yb, xb) u8
    ac_strategy: np.ndarray   # (yb, xb) u8, (raw << 1) | first
    ytox: np.ndarray          # (ty, tx) i8
    ytob: np.ndarray
    quant_dc: np.ndarray      # (3, yb, xb) i16, X Y B
    coefficients: np.ndarray | None  # (yb, xb, 3, 64) i32
    num_nzeros: np.ndarray    # (3, yb, xb) u8
    tokens: np.ndarray | None  # (n, 2) u32: context, value (None when only the packed form was asked for)
    group_offsets: np.ndarray  # (groups + 1,) u64
    histograms: np.ndarray    # (14850, 128) u32
    xyb: np.ndarray | None = None
    alpha: np.ndarray | None = None  # (h, w) u16 alpha after fringe clearing (RGBA input)
    packed_tokens: np.ndarray | None = None   # u32 words: the groups' storage form (AcTokens)
    packed_offsets: np.ndarray | None = None  # (groups + 1,) u64 word offsets


def ac_bits_estimate(result: "FrontendResult") -> float:
    """AC bits of a pass as an ideal coder would spend them on its tokens: the
    per-context symbol entropy of the histograms plus each token's raw bits
    (values >= 16 carry floor(log2 v) - 2 of them under the 4-2-0 hybrid
    split).  Context clustering and the headers are not counted, so this is a
    rate to compare passes by, not a file size."""
    h = result.histograms.astype(np.float64)
    tot = h.sum(axis=1, keepdims=True)
    p = np.divide(h, tot, out=np.ones_like(h), where=h > 0)
    bits = float(-(h * np.log2(p)).sum())
    if result.tokens is not None and len(result.tokens):
        v = result.tokens[:, 1].astype(np.int64)
        big = v[v >= 16]
        bits += float((np.floor(np.log2(big)) - 2).sum())
    return bits


# ORDER_SPECS (src/coeff_order.rs:117-125): the coefficients of each order
# slot (DCT8; the 8x8-sized transforms; 16x16; 32x32; 16x8 / 8x16; 32x8 /
# 8x32; 32x16 / 16x32); statistics and orders hold three channels of each
ORDER_SLOT_SIZES = (64, 64, 256, 1024, 128, 256, 512)
_ORDER_COUNTERS = 3 * sum(ORDER_SLOT_SIZES)


def _split_orders(flat: np.ndarray) -> list[np.ndarray]:
    out, off = [], 0
    for n in ORDER_SLOT_SIZES:
        out.append(flat[off:off + 3 * n].reshape(3, n).copy())
        off += 3 * n
    return out


def derive_orders(counts, blocks) -> tuple[int, list[np.ndarray], float]:
    """`derive_orders` (src/coeff_order.rs:621-673) on the host
    (jxg_derive_orders): from per-slot statistics, as
    `FrontendContext.order_stats` returns them, the used-order mask (bit =
    order group), per slot its (3, size) orders (scan position -> raw index,
    natural where not adopted) and the share of the expected scan walk the
    adopted orders remove."""
    flat = np.ascontiguousarray(np.concatenate([np.asarray(c, np.uint32).reshape(-1) for c in counts]))
    blk = np.ascontiguousarray(np.asarray(blocks, np.uint32))
    if flat.size != _ORDER_COUNTERS or blk.size != len(ORDER_SLOT_SIZES):
        raise EncodeError(100, "order statistics: one (3, size) array and one count per slot")
    orders = np.zeros(_ORDER_COUNTERS, np.uint32)
    used = ctypes.c_uint16()
    moved = ctypes.c_double()
    st = L.load().jxg_derive_orders(flat.ctypes.data, blk.ctypes.data, ctypes.byref(used),
                                    orders.ctypes.data, ctypes.byref(moved))
    if st:
        raise EncodeError(st, "jxg_derive_orders")
    return used.value, _split_orders(orders), moved.value


def _as_hwc(pixels: np.ndarray) -> np.ndarray:
    """(h, w) grey samples as (h, w, 1); other shapes unchanged."""
    pixels = np.ascontiguousarray(pixels)
    return pixels[:, :, None] if pixels.ndim == 2 else pixels


def _pixels_kind(pixels: np.ndarray, config: "EncodeConfig | None" = None) -> tuple[int, int]:
    if pixels.ndim != 3 or pixels.shape[2] not in (1, 2, 3, 4):
        raise EncodeError(9, f"expected (h, w, 1|2|3|4) samples, got {pixels.shape}")
    want = config.bits_per_sample if config is not None else 0
    if pixels.dtype == np.uint8:
        if want not in (0, 8):
            raise EncodeError(10, f"{want}-bit samples need uint16 words")
        return pixels.shape[2], 8
    if pixels.dtype == np.uint16:
        return pixels.shape[2], want if want else 16
    raise EncodeError(10, f"unsupported sample type {pixels.dtype}")


def _params_dict(p) -> dict:
    out = {n: getattr(p, n) for n, _ in L.FrameParams._fields_ if n != "reserved"}
    out["dc_step"] = list(p.dc_step)
    out["screen_content"] = bool(out["screen_content"])
    return out


def unpack_tokens(words: np.ndarray, word_offsets: np.ndarray,
                  group_offsets: np.ndarray) -> np.ndarray:
    """(n, 2) context/value tokens from the groups' storage form
    (AcToken::unpack, src/entropy/token_stream.rs:44-48): a group with as
    many words as tokens is packed (context << 18 | value), one with twice
    as many holds (context, value) pairs."""
    out = np.zeros((int(group_offsets[-1] - group_offsets[0]), 2), np.uint32)
    base = int(group_offsets[0])
    for g in range(len(group_offsets) - 1):
        t0, t1 = int(group_offsets[g]) - base, int(group_offsets[g + 1]) - base
        w0, w1 = int(word_offsets[g]), int(word_offsets[g + 1])
        w = words[w0:w1]
        if w1 - w0 == t1 - t0:
            out[t0:t1, 0] = w >> 18
            out[t0:t1, 1] = w & 0x3FFFF
        elif w1 - w0 == 2 * (t1 - t0):
            out[t0:t1] = w.reshape(-1, 2)
        else:
            raise ValueError(f"group {g}: {w1 - w0} words for {t1 - t0} tokens")
    return out


def _result_buffers(p: dict, width: int, height: int, coefficients: bool, xyb: bool,
                    alpha: bool = False, packed: bool = False):
    """Host arrays for every output of one frame and the C struct pointing at them."""
    fi = frame_info(width, height)
    xb, yb = fi.xsize_blocks, fi.ysize_blocks
    r = FrontendResult(
        params=p,
        quant_field=np.zeros((yb, xb), np.uint8),
        ac_strategy=np.zeros((yb, xb), np.uint8),
        ytox=np.zeros((fi.ysize_tiles, fi.xsize_tiles), np.int8),
        ytob=np.zeros((fi.ysize_tiles, fi.xsize_tiles), np.int8),
        quant_dc=np.zeros((3, yb, xb), np.int16),
        coefficients=np.zeros((yb, xb, 3, 64), np.int32) if coefficients else None,
        num_nzeros=np.zeros((3, yb, xb), np.uint8),
        tokens=np.zeros((max(int(p["num_tokens"]), 1), 2), np.uint32),
        group_offsets=np.zeros(fi.num_groups + 1, np.uint64),
        histograms=np.zeros((L.NUM_FINE_AC_CONTEXTS, L.ALPHABET_SIZE), np.uint32),
        xyb=np.zeros((3, height, width), np.float32) if xyb else None,
        alpha=np.zeros((height, width), np.uint16) if alpha else None,
        packed_tokens=np.zeros(max(2 * int(p["num_tokens"]), 1), np.uint32) if packed else None,
        packed_offsets=np.zeros(fi.num_groups + 1, np.uint64) if packed else None,
    )
    o = L.FrontendOutput()
    o.quant_field = r.quant_field.ctypes.data
    o.ac_strategy = r.ac_strategy.ctypes.data
    o.ytox_map = r.ytox.ctypes.data
    o.ytob_map = r.ytob.ctypes.data
    o.quant_dc = r.quant_dc.ctypes.data
    o.coefficients = r.coefficients.ctypes.data if coefficients else None
    o.num_nzeros = r.num_nzeros.ctypes.data
    o.xyb = r.xyb.ctypes.data if xyb else None
    o.tokens = r.tokens.ctypes.data
    o.token_capacity = r.tokens.shape[0]
    o.group_offsets = r.group_offsets.ctypes.data
    o.histograms = r.histograms.ctypes.data
    o.alpha = r.alpha.ctypes.data if alpha else None
    if packed:
        o.packed_tokens = r.packed_tokens.ctypes.data
        o.packed_capacity = r.packed_tokens.shape[0]
        o.packed_offsets = r.packed_offsets.ctypes.data
    return r, o


def _trim(r: FrontendResult) -> FrontendResult:
    r.tokens = r.tokens[: int(r.params["num_tokens"])]
    if r.packed_tokens is not None:
        r.packed_tokens = r.packed_tokens[: int(r.packed_offsets[-1])]
    return r


class FrontendContext:
    """One device encoder (`EncodingContext`, src/encoding_context.rs:609)."""

    def __init__(self, device: int = 0):
        self._lib = L.load()
        self._ctx = ctypes.c_void_p()
        st = self._lib.jxg_context_create(device, ctypes.byref(self._ctx))
        if st:
            raise EncodeError(st, "could not create a CUDA context for the front end")

    def close(self):
        if self._ctx:
            self._lib.jxg_context_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st:
            msg = self._lib.jxg_context_last_error(self._ctx)
            raise EncodeError(st, msg.decode() if msg else "")

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._ctx

    def set_stream(self, stream_ptr: int | None):
        """Launch on `stream_ptr` (a cudaStream_t); None or 0 restores the
        context's own stream (the legacy default stream cannot be selected)."""
        self._check(self._lib.jxg_context_set_stream(self._ctx, stream_ptr or None))

    def run(self, pixels: np.ndarray, config: EncodeConfig):
        """Host input: copy in, run, wait (jxg_frontend_run)."""
        pixels = _as_hwc(pixels)
        ch, bits = _pixels_kind(pixels, config)
        h, w = pixels.shape[:2]
        cfg = config._c()
        self._check(self._lib.jxg_frontend_run(self._ctx, pixels.ctypes.data, w, h, ch, bits,
                                               ctypes.byref(cfg)))

    def run_device(self, device_ptr: int, width: int, height: int, channels: int, bits: int,
                   config: EncodeConfig):
        """Device input: enqueue only (jxg_frontend_run_device)."""
        cfg = config._c()
        self._check(self._lib.jxg_frontend_run_device(self._ctx, device_ptr, width, height,
                                                      channels, bits, ctypes.byref(cfg)))

    def params(self) -> dict:
        p = L.FrameParams()
        self._check(self._lib.jxg_frontend_params(self._ctx, ctypes.byref(p)))
        return _params_dict(p)

    def fetch(self, width: int, height: int, *, coefficients: bool = True,
              xyb: bool = False, alpha: bool = False, packed: bool = False) -> FrontendResult:
        p = self.params()
        r, o = _result_buffers(p, width, height, coefficients, xyb, alpha, packed)
        self._check(self._lib.jxg_frontend_fetch(self._ctx, ctypes.byref(o)))
        return _trim(r)

    def enqueue(self, pixels: np.ndarray, config: EncodeConfig, out: "PinnedOutputs"):
        """Asynchronous front end (jxg_frontend_enqueue): `pixels` and `out`
        should be pinned; call wait() before reading `out`."""
        ch, bits = _pixels_kind(pixels, config)
        h, w = pixels.shape[:2]
        cfg = config._c()
        self._check(self._lib.jxg_frontend_enqueue(self._ctx, pixels.ctypes.data, w, h, ch, bits,
                                                   ctypes.byref(cfg), ctypes.byref(out.params),
                                                   ctypes.byref(out.c)))

    def wait(self):
        self._check(self._lib.jxg_frontend_wait(self._ctx))

    def pixel_chromacity(self) -> tuple[np.ndarray, int, int]:
        """pixel_chromacity_steps (src/frame/chroma.rs:89-165) on the last
        pass's XYB (jxg_pixel_chromacity): the seven counts (X steps at three
        levels, B - Y steps at three, exposed blue) and the extra X and B
        quant-scale steps."""
        counts = np.zeros(7, np.uint32)
        xs, bs = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self._lib.jxg_pixel_chromacity(self._ctx, counts.ctypes.data, ctypes.byref(xs),
                                                   ctypes.byref(bs)))
        return counts, xs.value, bs.value

    def order_stats(self) -> tuple[list[np.ndarray], np.ndarray]:
        """The coefficient-order statistics of the last pass's first frame
        (jxg_order_stats): per order slot a (3, size) u32 array of the
        transforms whose level is non-zero at each raw index, and the
        transforms per slot."""
        counts = np.zeros(_ORDER_COUNTERS, np.uint32)
        blocks = np.zeros(len(ORDER_SLOT_SIZES), np.uint32)
        self._check(self._lib.jxg_order_stats(self._ctx, counts.ctypes.data, blocks.ctypes.data))
        return _split_orders(counts), blocks

    def batch(self, pixels_on_device: bool = False) -> "FrontendBatch":
        """A batch of frames run as one pass on this context."""
        return FrontendBatch(self, pixels_on_device)

    def frontend(self, pixels: np.ndarray, config: EncodeConfig, *, coefficients: bool = True,
                 xyb: bool = False, packed: bool = False) -> FrontendResult:
        pixels = _as_hwc(pixels)
        self.run(pixels, config)
        return self.fetch(pixels.shape[1], pixels.shape[0], coefficients=coefficients, xyb=xyb,
                          alpha=pixels.shape[2] in (2, 4), packed=packed)

    # operator table -----------------------------------------------------
    def chroma_hf_protection(self, xyb: np.ndarray, distance: float, field: np.ndarray) -> np.ndarray:
        """apply_chroma_hf_protection (src/adaptive_quant.rs:303-402) of (3, h, w)
        XYB planes on a copy of the (yb, xb) u8 field (jxg_op_chroma_hf_protection)."""
        xyb = np.ascontiguousarray(xyb, np.float32)
        _, h, w = xyb.shape
        out = np.ascontiguousarray(field, np.uint8).copy()
        self._check(self._lib.jxg_op_chroma_hf_protection(self._ctx, xyb.ctypes.data, w, h,
                                                          float(distance), out.ctypes.data))
        return out

    def fill_quant_field(self, xyb: np.ndarray, distance: float, inv_scale: float) -> np.ndarray:
        xyb = np.ascontiguousarray(xyb, np.float32)
        _, h, w = xyb.shape
        fi = frame_info(w, h)
        out = np.zeros((fi.ysize_blocks, fi.xsize_blocks), np.uint8)
        self._check(self._lib.jxg_op_fill_quant_field(self._ctx, xyb.ctypes.data, w, h, distance,
                                                      inv_scale, out.ctypes.data))
        return out

    def gaborish_inverse(self, xyb: np.ndarray, mul: float = 0.9908511) -> np.ndarray:
        """gaborish_inverse (src/gaborish.rs:44) of (3, h, w) planes."""
        x = np.ascontiguousarray(xyb, np.float32)
        out = np.zeros_like(x)
        self._check(self._lib.jxg_op_gaborish_inverse(self._ctx, x.ctypes.data, x.shape[2],
                                                      x.shape[1], mul, out.ctypes.data))
        return out

    def gaborish(self, xyb: np.ndarray) -> np.ndarray:
        """The decoder's Gaborish (src/epf_filter.rs:165) of (3, h, w) planes."""
        x = np.ascontiguousarray(xyb, np.float32)
        out = np.zeros_like(x)
        self._check(self._lib.jxg_op_gaborish(self._ctx, x.ctypes.data, x.shape[2], x.shape[1],
                                              out.ctypes.data))
        return out

    def epf(self, xyb: np.ndarray, sigma_quant: np.ndarray, iters: int, quant_mul: float = 0.46,
            pass0: float = 0.9, pass2: float = 6.5, border_mul: float = 2.0 / 3.0,
            channel_scale=(40.0, 5.0, 3.5), sharpness: int = 7) -> np.ndarray:
        """jxg_op_epf: the decoder's edge-preserving filter over (3, h, w)
        planes with one sigma_quant value per 8x8 block."""
        x = np.ascontiguousarray(xyb, np.float32)
        _, h, w = x.shape
        sq = np.ascontiguousarray(sigma_quant, np.float32)
        if sq.size != ((w + 7) // 8) * ((h + 7) // 8):
            raise EncodeError(100, "one sigma_quant value per 8x8 block")
        cs = np.ascontiguousarray(channel_scale, np.float32)
        out = np.zeros_like(x)
        self._check(self._lib.jxg_op_epf(self._ctx, x.ctypes.data, w, h, sq.ctypes.data, iters, quant_mul,
                                         pass0, pass2, border_mul, cs.ctypes.data, sharpness, out.ctypes.data))
        return out

    def luma_proxy(self, source: np.ndarray, test: np.ndarray) -> tuple[float, np.ndarray]:
        """jxg_op_luma_proxy: the reference's six-term luma proxy of `test`
        against `source` ((h, w) Y planes): (score, the six terms)."""
        a = np.ascontiguousarray(source, np.float32)
        b = np.ascontiguousarray(test, np.float32)
        if a.shape != b.shape or a.ndim != 2:
            raise EncodeError(100, "two (h, w) planes of one size")
        score = ctypes.c_double()
        terms = np.zeros(6, np.float64)
        self._check(self._lib.jxg_op_luma_proxy(self._ctx, a.ctypes.data, b.ctypes.data, a.shape[1], a.shape[0],
                                                ctypes.byref(score), terms.ctypes.data))
        return score.value, terms

    def epf_fit(self, source_y: np.ndarray, recon: np.ndarray, sigma_quant: np.ndarray, distance: float,
                baseline=(2, None, None, 7)):
        """jxg_op_epf_fit: the encoder's EPF fit over a reconstruction;
        baseline and result as (iters, quant_mul or None, pass0 or None,
        sharpness); returns (choice, its proxy score)."""
        y = np.ascontiguousarray(source_y, np.float32)
        r = np.ascontiguousarray(recon, np.float32)
        h, w = y.shape
        if r.shape != (3, h, w):
            raise EncodeError(100, "recon must be (3, h, w) like source_y")
        sq = np.ascontiguousarray(sigma_quant, np.float32)
        if sq.size != ((w + 7) // 8) * ((h + 7) // 8):
            raise EncodeError(100, "one sigma_quant value per 8x8 block")
        ch = np.array([baseline[0], np.nan if baseline[1] is None else baseline[1],
                       np.nan if baseline[2] is None else baseline[2], baseline[3]], np.float32)
        score = ctypes.c_double()
        self._check(self._lib.jxg_op_epf_fit(self._ctx, y.ctypes.data, r.ctypes.data, w, h, sq.ctypes.data,
                                             distance, ch.ctypes.data, ctypes.byref(score)))
        opt = lambda v: None if np.isnan(v) else float(v)  # noqa: E731
        return (int(ch[0]), opt(ch[1]), opt(ch[2]), int(ch[3])), score.value

    def dct8x8(self, blocks: np.ndarray) -> np.ndarray:
        blocks = np.ascontiguousarray(blocks, np.float32).reshape(-1, 64)
        out = np.zeros_like(blocks)
        self._check(self._lib.jxg_op_dct8x8(self._ctx, blocks.ctypes.data, blocks.shape[0],
                                            out.ctypes.data))
        return out

    DCT_KINDS = {"8x8": (0, 8, 8, 1), "8x16": (1, 16, 8, 2), "16x8": (2, 8, 16, 2),
                 "16x16": (3, 16, 16, 4), "16x32": (4, 32, 16, 8), "32x16": (5, 16, 32, 8),
                 "32x32": (6, 32, 32, 16), "32x8": (7, 8, 32, 4), "8x32": (8, 32, 8, 4),
                 "64x64": (9, 64, 64, 64), "64x32": (10, 32, 64, 32), "32x64": (11, 64, 32, 32),
                 "128x128": (12, 128, 128, 256), "128x64": (13, 64, 128, 128),
                 "64x128": (14, 128, 64, 128)}

    def dct(self, name: str, blocks: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """DctFn<W, H, N> (src/dct.rs) of (count, H, W) blocks named rows x
        columns as the reference does ("8x16" = 8 rows of 16): (count, W H)
        coefficients and (count, D) DC values of the covered 8x8 blocks."""
        kind, w, h, ndc = self.DCT_KINDS[name]
        b = np.ascontiguousarray(blocks, np.float32).reshape(-1, h * w)
        out = np.zeros_like(b)
        dc = np.zeros((b.shape[0], ndc), np.float32)
        self._check(self._lib.jxg_op_dct(self._ctx, kind, b.ctypes.data, b.shape[0],
                                         out.ctypes.data, dc.ctypes.data))
        return out, dc

    def idct(self, name: str, coefficients: np.ndarray) -> np.ndarray:
        """The inverse of `dct` (IdctMethods, src/dct.rs:358): (count, H, W) samples."""
        kind, w, h, _ = self.DCT_KINDS[name]
        c = np.ascontiguousarray(coefficients, np.float32).reshape(-1, h * w)
        out = np.zeros_like(c)
        self._check(self._lib.jxg_op_idct(self._ctx, kind, c.ctypes.data, c.shape[0],
                                          out.ctypes.data))
        return out.reshape(-1, h, w)

    SMALL_TRANSFORMS = {"identity": 0, "dct2x2": 1, "dct4x4": 2, "dct4x8": 3, "dct8x4": 4,
                        "inv_identity": 5, "inv_dct2x2": 6,
                        "afv0": 7, "afv1": 8, "afv2": 9, "afv3": 10}

    def small_transform(self, name: str, blocks: np.ndarray) -> np.ndarray:
        """The 8x8-sized transforms besides DCT8 (identity8x8, dct2x2_8x8,
        dct4x4, dct4x8, dct8x4 and the identity / DCT2x2 inverses, src/dct.rs;
        afv_from_pixels kinds 0..3, src/afv.rs:207) of (count, 8, 8) blocks:
        (count, 64)."""
        b = np.ascontiguousarray(blocks, np.float32).reshape(-1, 64)
        out = np.zeros_like(b)
        self._check(self._lib.jxg_op_small_transform(self._ctx, self.SMALL_TRANSFORMS[name],
                                                     b.ctypes.data, b.shape[0], out.ctypes.data))
        return out

    def pack_tokens(self, tokens: np.ndarray, group_offsets: np.ndarray
                    ) -> tuple[np.ndarray, np.ndarray]:
        """AcTokens::from per group (src/entropy/token_stream.rs:59-76) on the
        device: (words, word offsets) of the groups' storage form."""
        tokens = np.ascontiguousarray(tokens, np.uint32).reshape(-1, 2)
        goffs = np.ascontiguousarray(group_offsets, np.uint64)
        n = int(goffs[-1] - goffs[0])
        words = np.zeros(max(2 * n, 1), np.uint32)
        woffs = np.zeros(goffs.shape[0], np.uint64)
        self._check(self._lib.jxg_op_pack_tokens(
            self._ctx, tokens.ctypes.data if tokens.size else None, goffs.ctypes.data,
            goffs.shape[0] - 1, words.ctypes.data, words.shape[0], woffs.ctypes.data))
        return words[: int(woffs[-1])], woffs

    # quant-field refinement ----------------------------------------------------
    def refine_begin(self) -> tuple[int, int]:
        """jxg_refine_begin: refine the frame of the last (UltraFast) pass;
        returns its block grid (xsize_blocks, ysize_blocks)."""
        w, h = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._lib.jxg_refine_begin(self._ctx, ctypes.byref(w), ctypes.byref(h)))
        self._refine_size = (w.value, h.value)
        self._refine_blocks = ((w.value + 7) // 8, (h.value + 7) // 8)
        return self._refine_blocks

    def refine_eval(self, rate_lambda: float, theta_ptr: int | None = None, grad_ptr: int | None = None,
                    levels: bool = False):
        """jxg_refine_eval at device `theta_ptr` (None: the context's own
        theta): ((loss, distortion, bits), levels or None); d loss / d theta
        into device `grad_ptr` when given.  Levels are (blocks, 3, 64) in raw
        order."""
        loss = np.zeros(3, np.float64)
        lv = None
        if levels:
            xb, yb = self._refine_blocks
            lv = np.zeros((xb * yb, 3, 64), np.int32)
        self._check(self._lib.jxg_refine_eval(self._ctx, theta_ptr, rate_lambda, grad_ptr,
                                              loss.ctypes.data, None if lv is None else lv.ctypes.data))
        return (float(loss[0]), float(loss[1]), float(loss[2])), lv

    def refine_weights(self, ssim: float = 1.0, proxy: float = 0.1):
        """jxg_refine_set_weights: distortion = ssim x (1 - SSIM) + proxy x the
        reference's luma proxy."""
        self._check(self._lib.jxg_refine_set_weights(self._ctx, ssim, proxy))
        self._refine_weights = (float(ssim), float(proxy))

    @property
    def refine_weights_now(self) -> tuple[float, float]:
        return getattr(self, "_refine_weights", (1.0, 0.1))

    def refine_step(self, rate_lambda: float, learning_rate: float) -> tuple[float, float, float]:
        """One Adam step on the context's theta; the loss before it."""
        loss = np.zeros(3, np.float64)
        self._check(self._lib.jxg_refine_step(self._ctx, rate_lambda, learning_rate, loss.ctypes.data))
        return float(loss[0]), float(loss[1]), float(loss[2])

    def refine_theta(self, theta: np.ndarray | None = None) -> np.ndarray:
        """The context's theta as (yb, xb) floats; with `theta`, set it first."""
        xb, yb = self._refine_blocks
        if theta is not None:
            t = np.ascontiguousarray(theta, np.float32).reshape(-1)
            if t.size != xb * yb:
                raise EncodeError(100, f"theta needs {xb * yb} values")
            self._check(self._lib.jxg_refine_theta(self._ctx, t.ctypes.data, 1))
        out = np.zeros((yb, xb), np.float32)
        self._check(self._lib.jxg_refine_theta(self._ctx, out.ctypes.data, 0))
        return out

    def refine_decoded(self, theta_ptr: int | None = None) -> np.ndarray:
        """The model's decoded XYB planes (3, h, w) at theta (the context's own
        by default): dequantised, inverse-transformed, decoded DC, EPF."""
        if not hasattr(self, "_refine_size"):
            raise EncodeError(100, "refine_begin first")
        w, h = self._refine_size
        out = np.zeros((3, h, w), np.float32)
        self._check(self._lib.jxg_refine_decoded(self._ctx, theta_ptr, out.ctypes.data))
        return out

    def refine_field(self, theta_ptr: int | None = None) -> np.ndarray:
        """round(qf * exp(theta)) in 1..255 as a (yb, xb) uint8 array."""
        xb, yb = self._refine_blocks
        out = np.zeros((yb, xb), np.uint8)
        self._check(self._lib.jxg_refine_field(self._ctx, theta_ptr, out.ctypes.data))
        return out

    def refine_rate_slope(self, pixels: int, delta: float = 0.1) -> float:
        """-dD / d(bits per pixel) of a uniform change of theta by +-delta
        around the context's theta: the lambda at which the frame's overall
        rate is, to first order, where the pass put it (pixels = width *
        height of the frame)."""
        t = self.refine_theta()
        self.refine_theta(t + delta)
        (_, d_hi, b_hi), _ = self.refine_eval(0.0)
        self.refine_theta(t - delta)
        (_, d_lo, b_lo), _ = self.refine_eval(0.0)
        self.refine_theta(t)
        if b_hi == b_lo:
            return 0.0
        return max(0.0, -(d_hi - d_lo) / ((b_hi - b_lo) / pixels))

    def refine(self, steps: int = 8, rate_lambda: float = 0.002, learning_rate: float = 0.05,
               monotone: bool = True):
        """Refine the last pass's quant field: `steps` Adam steps from theta = 0.
        With `monotone`, a step whose rounded loss is higher than the loss
        before it is taken back and the learning rate halved (Adam restarts
        there), so the loss never rises.  Returns (field (yb, xb) uint8,
        the loss before each step, the final loss)."""
        self.refine_begin()
        current, _ = self.refine_eval(rate_lambda)
        history = []
        lr = learning_rate
        for _ in range(steps):
            history.append(current)
            before = self.refine_theta() if monotone else None
            self.refine_step(rate_lambda, lr)
            after, _ = self.refine_eval(rate_lambda)
            if monotone and after[0] > current[0]:
                self.refine_theta(before)
                lr *= 0.5
            else:
                current = after
        return self.refine_field(), history, current

    def refine_model(self) -> dict:
        """The model's constants, source coefficients, inverse transform and
        decoded DC."""
        xb, yb = self._refine_blocks
        nb = xb * yb
        k = np.zeros(414, np.float32)
        coef = np.zeros((nb, 3, 64), np.float32)
        inv = np.zeros((64, 64), np.float32)
        dc = np.zeros((nb, 3), np.float32)
        self._check(self._lib.jxg_refine_model(self._ctx, k.ctypes.data, coef.ctypes.data,
                                               inv.ctypes.data, dc.ctypes.data))
        return {"scale": float(k[0]), "qm_mul": k[1:4].copy(), "matrix": k[4:196].reshape(3, 64).copy(),
                "inv_matrix": k[196:388].reshape(3, 64).copy(), "thresholds": k[388:400].reshape(3, 4).copy(),
                "epf": {"stages": [(int(k[401 + i]), float(k[404 + i])) for i in range(int(k[400]))],
                        "border": float(k[407]), "channel_scale": k[408:411].copy(),
                        "quant_mul": float(k[411]), "lut": float(k[412]), "quant_scale": float(k[413])},
                "coef": coef, "inverse": inv, "dc": dc}

    def run_with_field(self, pixels: np.ndarray, config: EncodeConfig, quant_field: np.ndarray):
        """jxg_frontend_run_with_field, host pixels and a host (yb, xb) field."""
        pixels = _as_hwc(pixels)
        ch, bits = _pixels_kind(pixels, config)
        h, w = pixels.shape[:2]
        fi = frame_info(w, h)
        qf = np.ascontiguousarray(quant_field, np.uint8)
        if qf.shape != (fi.ysize_blocks, fi.xsize_blocks):
            raise EncodeError(100, f"the field must be ({fi.ysize_blocks}, {fi.xsize_blocks})")
        cfg = config._c()
        self._check(self._lib.jxg_frontend_run_with_field(self._ctx, pixels.ctypes.data, w, h, ch, bits,
                                                          ctypes.byref(cfg), qf.ctypes.data, 0))

    def frontend_with_field(self, pixels: np.ndarray, config: EncodeConfig, quant_field: np.ndarray,
                            **kw) -> FrontendResult:
        pixels = _as_hwc(pixels)
        self.run_with_field(pixels, config, quant_field)
        return self.fetch(pixels.shape[1], pixels.shape[0], alpha=pixels.shape[2] in (2, 4), **kw)

    # launch geometry and its autotuner --------------------------------------
    TUNE_KERNELS = ("k_cost_dct8", "k_cost_16x8", "k_cost_8x16", "k_cost_16x16", "k_layout_dct8",
                    "k_layout_16x8", "k_layout_8x16", "k_layout_16x16", "k_retile", "k_site")

    def launch_geometry(self) -> dict:
        """Warps per CTA of each tunable Speed::Fastest kernel."""
        w = (ctypes.c_uint8 * len(self.TUNE_KERNELS))()
        self._check(self._lib.jxg_get_launch_geometry(self._ctx, w))
        return dict(zip(self.TUNE_KERNELS, list(w)))

    def set_launch_geometry(self, geometry: dict):
        cur = self.launch_geometry()
        cur.update(geometry)
        w = (ctypes.c_uint8 * len(self.TUNE_KERNELS))(*[cur[k] for k in self.TUNE_KERNELS])
        self._check(self._lib.jxg_set_launch_geometry(self._ctx, w))

    def autotune(self, device_ptr: int, width: int, height: int, channels: int, bits: int,
                 config: EncodeConfig, rounds: int = 2) -> tuple[dict, dict]:
        """jxg_autotune on a frame in device memory: the chosen geometry and
        every candidate's average launch time {kernel: {warps: ms}}."""
        times = np.full(len(self.TUNE_KERNELS) * 4, np.nan, np.float64)
        cfg = config._c()
        self._check(self._lib.jxg_autotune(self._ctx, device_ptr, width, height, channels, bits,
                                           ctypes.byref(cfg), rounds, times.ctypes.data))
        t = {k: {w: float(times[i * 4 + j]) for j, w in enumerate((1, 2, 4, 8))}
             for i, k in enumerate(self.TUNE_KERNELS)}
        return self.launch_geometry(), t

    # timing -------------------------------------------------------------
    def enable_kernel_timing(self, on: bool = True):
        self._check(self._lib.jxg_enable_kernel_timing(self._ctx, 1 if on else 0))

    def kernel_times(self) -> dict:
        cap = 64
        names = (ctypes.c_char_p * cap)()
        ms = (ctypes.c_double * cap)()
        cnt = (ctypes.c_uint64 * cap)()
        n = self._lib.jxg_kernel_times(self._ctx, names, ms, cnt, cap)
        if n < 0:
            self._check(n)
        return {names[i].decode(): (ms[i], cnt[i]) for i in range(min(n, cap))}

    def reset_kernel_times(self):
        self._check(self._lib.jxg_reset_kernel_times(self._ctx))


class PinnedOutputs:
    """Pinned host buffers for every output of one width x height frame, for
    FrontendContext.enqueue (allocated with torch's pinned allocator).  With
    `packed` the tokens come in the groups' storage form only (one word per
    token unless a group holds values of 2^18 or more; room for max_tokens
    words)."""

    def __init__(self, width: int, height: int, *, channels: int = 3, coefficients: bool = False,
                 xyb: bool = False, packed: bool = False):
        import torch

        fi = frame_info(width, height)
        xb, yb = fi.xsize_blocks, fi.ysize_blocks
        nb, nt = xb * yb, fi.xsize_tiles * fi.ysize_tiles

        def pin(shape, dt):
            return torch.empty(shape, dtype=dt, pin_memory=True).numpy()

        self.width, self.height, self.info = width, height, fi
        self.quant_field = pin((yb, xb), torch.uint8)
        self.ac_strategy = pin((yb, xb), torch.uint8)
        self.ytox = pin((fi.ysize_tiles, fi.xsize_tiles), torch.int8)
        self.ytob = pin((fi.ysize_tiles, fi.xsize_tiles), torch.int8)
        self.quant_dc = pin((3, yb, xb), torch.int16)
        self.coefficients = pin((yb, xb, 3, 64), torch.int32) if coefficients else None
        self.num_nzeros = pin((3, yb, xb), torch.uint8)
        self.tokens = None if packed else pin((fi.max_tokens, 2), torch.int32).view(np.uint32)
        self.packed_tokens = pin((fi.max_tokens,), torch.int32).view(np.uint32) if packed else None
        self.packed_offsets = (pin((fi.num_groups + 1,), torch.int64).view(np.uint64)
                               if packed else None)
        self.group_offsets = pin((fi.num_groups + 1,), torch.int64).view(np.uint64)
        self.histograms = pin((L.NUM_FINE_AC_CONTEXTS, L.ALPHABET_SIZE), torch.int32).view(np.uint32)
        self.xyb = pin((3, height, width), torch.float32) if xyb else None
        self.alpha = pin((height, width), torch.int16).view(np.uint16) if channels in (2, 4) else None
        self.params = L.FrameParams()
        o = L.FrontendOutput()
        o.quant_field = self.quant_field.ctypes.data
        o.ac_strategy = self.ac_strategy.ctypes.data
        o.ytox_map = self.ytox.ctypes.data
        o.ytob_map = self.ytob.ctypes.data
        o.quant_dc = self.quant_dc.ctypes.data
        o.coefficients = self.coefficients.ctypes.data if coefficients else None
        o.num_nzeros = self.num_nzeros.ctypes.data
        o.xyb = self.xyb.ctypes.data if xyb else None
        if packed:
            o.packed_tokens = self.packed_tokens.ctypes.data
            o.packed_capacity = fi.max_tokens
            o.packed_offsets = self.packed_offsets.ctypes.data
        else:
            o.tokens = self.tokens.ctypes.data
            o.token_capacity = fi.max_tokens
        o.group_offsets = self.group_offsets.ctypes.data
        o.histograms = self.histograms.ctypes.data
        o.alpha = self.alpha.ctypes.data if self.alpha is not None else None
        self.c = o

    def result(self) -> FrontendResult:
        """Copies of the outputs after FrontendContext.wait()."""
        p = _params_dict(self.params)
        n = int(p["num_tokens"])
        return FrontendResult(
            params=p, quant_field=self.quant_field.copy(), ac_strategy=self.ac_strategy.copy(),
            ytox=self.ytox.copy(), ytob=self.ytob.copy(), quant_dc=self.quant_dc.copy(),
            coefficients=None if self.coefficients is None else self.coefficients.copy(),
            num_nzeros=self.num_nzeros.copy(),
            tokens=None if self.tokens is None else self.tokens[:n].copy(),
            group_offsets=self.group_offsets.copy(), histograms=self.histograms.copy(),
            xyb=None if self.xyb is None else self.xyb.copy(),
            alpha=None if self.alpha is None else self.alpha.copy(),
            packed_tokens=(None if self.packed_tokens is None
                           else self.packed_tokens[: int(self.packed_offsets[-1])].copy()),
            packed_offsets=None if self.packed_offsets is None else self.packed_offsets.copy())


class FrontendBatch:
    """Many frames in one pass (jxg_batch_*): one launch per stage over all
    frames, optionally recorded as a CUDA graph and replayed.  The pixel
    arrays (or device pointers) handed to `add` are kept referenced and read
    again at every `run`."""

    def __init__(self, ctx: FrontendContext, pixels_on_device: bool = False):
        self._ctx = ctx
        self._lib = ctx._lib
        self._b = ctypes.c_void_p()
        self._keep = []
        self._sizes = []
        self._check(self._lib.jxg_batch_create(ctx.handle, 1 if pixels_on_device else 0,
                                               ctypes.byref(self._b)))

    def _check(self, st: int):
        self._ctx._check(st)

    def close(self):
        if self._b:
            self._lib.jxg_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self._sizes)

    def add(self, pixels: np.ndarray, config: EncodeConfig) -> int:
        pixels = _as_hwc(pixels)
        ch, bits = _pixels_kind(pixels, config)
        h, w = pixels.shape[:2]
        return self._add(pixels.ctypes.data, w, h, ch, bits, config, pixels)

    def add_device(self, device_ptr: int, width: int, height: int, channels: int, bits: int,
                   config: EncodeConfig, keep=None) -> int:
        return self._add(device_ptr, width, height, channels, bits, config, keep)

    def _add(self, ptr, w, h, ch, bits, config, keep) -> int:
        cfg = config._c()
        idx = self._lib.jxg_batch_add(self._b, ptr, w, h, ch, bits, ctypes.byref(cfg))
        if idx < 0:
            self._check(-idx)
        self._keep.append(keep)
        self._sizes.append((w, h, ch))
        return idx

    def run(self, use_graph: bool = True):
        self._check(self._lib.jxg_batch_run(self._b, 1 if use_graph else 0))

    def params(self, index: int) -> dict:
        p = L.FrameParams()
        self._check(self._lib.jxg_batch_result(self._b, index, ctypes.byref(p), None))
        return _params_dict(p)

    def result(self, index: int, *, coefficients: bool = True, xyb: bool = False,
               packed: bool = False) -> FrontendResult:
        w, h, ch = self._sizes[index]
        p = self.params(index)
        r, o = _result_buffers(p, w, h, coefficients, xyb, ch in (2, 4), packed)
        self._check(self._lib.jxg_batch_result(self._b, index, None, ctypes.byref(o)))
        return _trim(r)


def encode_frontend(pixels: np.ndarray, config: EncodeConfig, device: int = 0, *,
                    refine_steps: int = 0, learning_rate: float = 0.05) -> FrontendResult:
    """One-shot front end: the device half of `encode_image` (src/encode_image.rs:1610).
    With `refine_steps` (UltraFast only), the pass's quant field is refined
    by that many monotone steps at the frame's own rate-distortion slope and
    the frame coded again with the refined field."""
    ctx = FrontendContext(device)
    try:
        res = ctx.frontend(pixels, config)
        if refine_steps <= 0:
            return res
        pixels = _as_hwc(pixels)
        ctx.refine_begin()
        lam = ctx.refine_rate_slope(pixels.shape[0] * pixels.shape[1])
        field, _, _ = ctx.refine(steps=refine_steps, rate_lambda=lam, learning_rate=learning_rate)
        return ctx.frontend_with_field(pixels, config, field)
    finally:
        ctx.close()
