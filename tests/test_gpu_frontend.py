"""Parity of the CUDA front end with the CPU oracle (bit-exact).

Every integer output must equal the oracle's: quant field, CfL maps, DC
levels, AC levels, non-zero counts, tokens, group offsets and histograms;
the XYB planes must match to the bit as well.
"""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic
from oracle import oracle as O
from tests.parity import assert_same, high_depth_image as _high_depth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def ultrafast(distance, transfer=J.TransferFunction.SRGB, bits=0):
    return J.EncodeConfig(distance=distance, speed=J.Speed.ULTRA_FAST, transfer=transfer,
                          bits_per_sample=bits)


def compare(ctx, img, distance, check_xyb=True, transfer=J.TransferFunction.SRGB, bits=0):
    want = O.frontend(img, distance, bits=bits or None, transfer=int(transfer))
    got = ctx.frontend(img, ultrafast(distance, transfer, bits), xyb=check_xyb)
    assert_same(got, want, check_xyb)
    return got, want


def test_config1_q90(ctx):
    compare(ctx, synthetic.config1_image(), 1.0)


@pytest.mark.parametrize("q", [0, 30, 50, 75, 85, 90, 94, 95, 98, 100])
def test_config1_qualities(ctx, q):
    compare(ctx, synthetic.config1_image(), J.distance_from_quality(q))


def test_full_contrast_at_minimum_distance(ctx):
    # full-swing 16-bit checker at the minimum distance: about the largest
    # levels the quantiser reaches (a few hundred, far inside the 16-bit
    # level store; wider levels would take its exact int32 side buffer)
    y, x = np.mgrid[0:96, 0:128]
    img = np.where(((x // 3) + (y // 5)) % 2 == 0, 65535, 0).astype(np.uint16)
    img = np.stack([img, 65535 - img, img // 2], axis=-1)
    got, _ = compare(ctx, img, 0.05)
    assert 100 < int(np.abs(got.coefficients).max()) < 32767


@pytest.mark.parametrize("w,h", [(1, 1), (7, 9), (27, 28), (33, 33), (64, 17), (65, 65),
                                 (257, 65), (300, 7), (255, 257)])
def test_ragged_sizes(ctx, w, h):
    img = synthetic.generate(w, h, 11 + w + h, rectangles=3)
    compare(ctx, img, 1.0)


@pytest.mark.parametrize("w,h", [(8, 2400), (2400, 8), (520, 264), (1032, 72)])
def test_token_chunks_of_partial_groups(ctx, w, h):
    # the tokenizer's chunks run through each group's blocks in token order:
    # one-block-wide and one-block-tall groups, odd partial groups at the
    # right and bottom edges, several chunks per row of groups
    img = synthetic.generate(w, h, 31 + w, rectangles=4)
    compare(ctx, img, 1.0, check_xyb=False)


def test_token_lookback_timeout_is_reported_and_the_context_stays_usable(ctx):
    from jixel_gb300 import _lib as L
    lib = L.load()
    assert lib.jxg_selftest_token_lookback(ctx.handle, 2000) == 102  # JXG_ERR_DEVICE_TIMEOUT
    compare(ctx, synthetic.generate(96, 64, 41), 1.0)


def test_multiple_dc_groups(ctx):
    img = synthetic.generate(2100, 300, 21, rectangles=30)
    compare(ctx, img, 1.5, check_xyb=False)


def test_rgba_and_sixteen_bit(ctx):
    compare(ctx, synthetic.generate(200, 120, 31, alpha=True), 1.0)
    compare(ctx, synthetic.generate(200, 120, 32, sixteen_bit=True), 1.45)
    compare(ctx, synthetic.generate(130, 70, 33, sixteen_bit=True, alpha=True), 2.0)


def test_screen_content_flat_image(ctx):
    img = np.zeros((128, 192, 3), np.uint8)
    img[:, :96] = (200, 30, 40)
    img[40:90, 100:180] = (10, 220, 90)
    got, want = compare(ctx, img, 1.0)
    assert got.params["screen_content"]


def test_fill_quant_field_operator(ctx):
    # the reference's own AQ fixture: src/adaptive_quant.rs:855-893
    for (w, h) in [(27, 28), (1, 1), (7, 9), (32, 32), (33, 33), (64, 17), (65, 65)]:
        y, x = np.mgrid[0:h, 0:w]
        xyb = np.stack([np.sin((x * 7 + y * 13 + c * 29).astype(np.float32) * np.float32(0.017))
                        .astype(np.float32) * np.float32(0.4) + np.float32(c * 0.05)
                        for c in range(3)]).astype(np.float32)
        got = ctx.fill_quant_field(xyb, 1.0, 1.0)
        # the oracle runs the same AQ through its front end on an XYB input
        want = oracle_aq(xyb, 1.0, 1.0)
        assert np.array_equal(got, want), (w, h)


def oracle_aq(xyb, distance, inv_scale):
    import ctypes
    _, h, w = xyb.shape
    xb, yb = (w + 7) // 8, (h + 7) // 8
    out = np.zeros((yb, xb), np.uint8)
    lib = O.lib()
    lib.orc_fill_quant_field_image.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                               ctypes.c_float, ctypes.c_float, ctypes.c_void_p]
    lib.orc_fill_quant_field_image(np.ascontiguousarray(xyb).ctypes.data, w, h, distance,
                                   inv_scale, out.ctypes.data)
    return out


def test_dct8x8_operator(ctx):
    rng = np.random.default_rng(3)
    blocks = rng.uniform(-1, 1, (257, 64)).astype(np.float32)
    got = ctx.dct8x8(blocks)
    want = np.stack([O.dct8x8(b) for b in blocks])
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_large_frame_invariants(ctx):
    img = synthetic.config2_image()
    got = ctx.frontend(img, ultrafast(1.0), coefficients=True)
    fi = J.frame_info(3840, 2160)
    # every block-channel emits its non-zero count; histograms count every token
    assert int(got.histograms.sum()) == got.tokens.shape[0]
    assert got.group_offsets[-1] == got.tokens.shape[0]
    assert np.all(np.diff(got.group_offsets.astype(np.int64)) >= 3)
    nz = (got.coefficients[..., 1:] != 0).sum(-1).transpose(2, 0, 1)
    assert np.array_equal(nz, got.num_nzeros)
    # the non-zero-count tokens carry exactly the stored counts, channel order Y, X, B
    assert got.quant_field.min() >= 1
    assert got.tokens[:, 0].max() < 14850
    # a full-frame oracle comparison on a 1/4 crop keeps the CPU time small
    crop = np.ascontiguousarray(img[:1080, :1920])
    compare(ctx, crop, 1.0, check_xyb=False)


@pytest.mark.parametrize("q", [75, 90, 95])
def test_config2_frames_whole(ctx, q):
    # the benchmarked 3840x2160 frame at each quality, every output compared
    compare(ctx, synthetic.config2_image(), J.distance_from_quality(q), check_xyb=False)


def test_invalid_inputs_raise(ctx):
    img = np.zeros((8, 8, 3), np.uint8)
    with pytest.raises(J.EncodeError) as e:
        ctx.run(img, J.EncodeConfig(distance=1.0, speed=J.Speed.FAST))
    assert e.value.variant == "Unsupported"
    with pytest.raises(J.EncodeError) as e:
        ctx.run(img, ultrafast(-1.0))
    assert e.value.variant == "InvalidDistance"
    with pytest.raises(J.EncodeError) as e:
        ctx.run(np.zeros((0, 8, 3), np.uint8), ultrafast(1.0))
    assert e.value.variant == "EmptyImage"
    # the context stays usable
    compare(ctx, synthetic.generate(40, 40, 5), 1.0)


def test_repeat_runs_are_identical(ctx):
    img = synthetic.generate(300, 200, 77)
    a = ctx.frontend(img, ultrafast(1.0))
    b = ctx.frontend(img, ultrafast(1.0))
    assert np.array_equal(a.tokens, b.tokens)
    assert np.array_equal(a.histograms, b.histograms)


@pytest.mark.parametrize("which,lo,hi", [
    (0, 0, 0x40000000),           # cube root: every float in [0, 2)
    (1, 0, 0x44800000),           # gamma ratio, inverted: [0, 1024)
    (2, 0, 0x44800000),           # gamma ratio, direct: [0, 1024)
    (3, 0, 0x3E4CCCCD + 1),       # masking square root: [0, 0.2]
    (4, 0, 0x40000000),           # cube root, packed two-lane path: [0, 2)
    (5, 0, 65536),                # 16-bit sample / 65535: every sample value
    (6, 0, 0x44800000),           # gamma ratio, inverted, packed two-lane path
    (7, 0, 0x44800000),           # gamma ratio, direct, packed two-lane path
    (8, 0, 0x3E4CCCCD + 1),       # masking square root, packed two-lane path
])
def test_fast_math_equals_ieee_on_every_input(ctx, which, lo, hi):
    # the fused sequences replacing IEEE division / sqrt on the hot paths give
    # bit-identical results on every input those paths can see
    import ctypes
    from jixel_gb300 import _lib as L
    lib = L.load()
    n = ctypes.c_uint64()
    first = ctypes.c_uint32()
    assert lib.jxg_selftest_math(ctx.handle, which, lo, hi, ctypes.byref(n), ctypes.byref(first)) == 0
    assert n.value == 0, hex(first.value)


def test_8192_square_rgb16_invariants(ctx):
    # the configs' largest frame: 8192x8192 RGB 16-bit linear at q85 (67 MP,
    # 1024 groups); size-independent checks on the whole frame, bit-exact
    # parity on a 2048x2048 crop
    img = synthetic.config5_image()
    d = J.distance_from_quality(85)
    lin = J.TransferFunction.LINEAR
    got = ctx.frontend(img, ultrafast(d, lin), coefficients=False)
    fi = J.frame_info(8192, 8192)
    assert fi.num_groups == 1024
    ntok = got.tokens.shape[0]
    assert int(got.histograms.sum()) == ntok == int(got.group_offsets[-1])
    # every block-channel emits at least its non-zero-count token
    assert np.all(np.diff(got.group_offsets.astype(np.int64)) >= 3 * 1024)
    # the non-zero counts add up to the non-zero coefficient tokens
    assert int((got.tokens[:, 1] != 0).sum()) >= int(got.num_nzeros.astype(np.int64).sum())
    assert got.quant_field.min() >= 1 and got.tokens[:, 0].max() < 14850
    crop = np.ascontiguousarray(img[2048:4096, 4096:6144])
    compare(ctx, crop, d, check_xyb=False, transfer=lin)


TF = J.TransferFunction


@pytest.mark.parametrize("bits,transfer", [
    (10, TF.SRGB), (12, TF.SRGB), (16, TF.SRGB), (10, TF.LINEAR), (16, TF.LINEAR),
    (12, TF.BT709), (16, TF.BT470M), (10, TF.BT470BG), (16, TF.SMPTE240), (12, TF.SMPTE428),
    (10, TF.BT2020_10BIT), (16, TF.UNSPECIFIED)])
def test_high_depth_transfers(ctx, bits, transfer):
    # encode_image_10bit / _12bit / _16bit with color_encoding.transfer:
    # every sample through TransferLut::build's table
    compare(ctx, _high_depth(150, 90, 40 + bits, bits), 1.0, transfer=transfer, bits=bits)


@pytest.mark.parametrize("bits", [10, 12])
def test_high_depth_alpha(ctx, bits):
    # encode_image_with_alpha_10bit / _12bit: alpha capped to the largest
    # code, then the fringe, fill and factors at that full scale
    compare(ctx, _high_depth(140, 100, 60 + bits, bits, alpha=True), 1.0, bits=bits)


@pytest.mark.parametrize("transfer", [TF.BT709, TF.LINEAR, TF.SMPTE428])
def test_eight_bit_with_other_transfers(ctx, transfer):
    # 8-bit samples outside the sRGB default decode with the f32 formula
    compare(ctx, synthetic.generate(120, 80, 70), 1.0, transfer=transfer)


def test_unsupported_transfers_and_depths(ctx):
    img = np.zeros((8, 8, 3), np.uint16)
    for tf, variant in ((TF.SMPTE2084, "Unsupported"), (TF.HLG, "Unsupported")):
        with pytest.raises(J.EncodeError) as e:
            ctx.run(img, ultrafast(1.0, tf))
        assert e.value.variant == variant
    with pytest.raises(J.EncodeError) as e:
        ctx.run(img, ultrafast(1.0, bits=9))
    assert e.value.variant == "BadBitDepth"
    compare(ctx, synthetic.generate(40, 40, 6), 1.0)


def _grey(w, h, seed, bits=8, alpha=False):
    img = synthetic.generate(w, h, seed, sixteen_bit=bits > 8, alpha=alpha)
    luma = img[..., 1]
    if bits not in (8, 16):
        luma = (luma.astype(np.uint32) * ((1 << bits) - 1) // 65535).astype(np.uint16)
    return np.stack([luma, img[..., 3]], axis=-1) if alpha else luma


@pytest.mark.parametrize("bits,alpha", [(8, False), (8, True), (10, False), (12, True), (16, False)])
def test_grey_input(ctx, bits, alpha):
    # encode_image_gray (+ _alpha, _10bit, _12bit, _16bit) on the lossy path:
    # the luma through the transfer table as R = G = B
    compare(ctx, _grey(130, 90, 80 + bits, bits, alpha), 1.0, bits=bits)
