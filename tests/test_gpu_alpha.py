"""RGBA frames: fringe clearing, invisible fill and alpha AQ factors on the
device against the oracle (bit-exact, alpha plane included).

The cases come from the reference's own alpha tests (src/alpha_fringe.rs,
src/invisible.rs, src/adaptive_quant.rs alpha_aq_tests) widened to whole
frames, plus the shapes the wavefront fill must get right: single rows and
columns, fully transparent frames, frames taller than one 1024-row group,
16-bit alpha, and the config-3 generator (radial ramp with transparent
discs).
"""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic
from oracle import oracle as O
from tests.parity import assert_same

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def ultrafast(distance):
    return J.EncodeConfig(distance=distance, speed=J.Speed.ULTRA_FAST)


def with_alpha(rgb, alpha):
    return np.ascontiguousarray(np.concatenate([rgb, alpha[..., None].astype(rgb.dtype)], axis=2))


def compare(ctx, img, distance=1.0):
    want = O.frontend(img, distance)
    got = ctx.frontend(img, ultrafast(distance), xyb=True)
    assert got.alpha is not None
    assert_same(got, want)
    return got, want


def test_fringe_cases_as_frames(ctx):
    # src/alpha_fringe.rs:233-299 planes as the alpha of whole frames
    rgb = synthetic.generate(64, 64, 41)
    a = np.zeros((64, 64), np.uint8)
    a[:, :20] = 255
    a[:, 20] = 3
    a[20:51, 40:] = 2
    got, _ = compare(ctx, with_alpha(rgb, a))
    assert np.all(got.alpha[:, 20] == 0) and got.alpha[35, 52] == 2
    y, x = np.mgrid[0:64, 0:64]
    b = np.where(y <= 7, 128, np.where((x + 2 * y) % 4 == 0, 254, 255)).astype(np.uint8)
    got, _ = compare(ctx, with_alpha(rgb, b))
    assert np.all(got.alpha[8:] == 255)  # the near-opaque sweep applied


def test_holes_fill_and_factors(ctx):
    for (w, h, seed) in [(1, 1, 51), (7, 9, 52), (64, 17, 53), (300, 200, 54), (513, 129, 55)]:
        compare(ctx, synthetic.generate(w, h, seed, alpha=True))


def test_single_rows_columns_and_transparent_frames(ctx):
    for (w, h) in [(97, 1), (1, 97), (40, 33)]:
        rgb = synthetic.generate(w, h, 60 + w)
        a = np.full((h, w), 255, np.uint8)
        a[:, ::3] = 0
        compare(ctx, with_alpha(rgb, a))
        compare(ctx, with_alpha(rgb, np.zeros((h, w), np.uint8)))


def test_taller_than_one_fill_group(ctx):
    # 2100 rows: three 1024-row wavefront groups, holes across the seams
    img = synthetic.generate(96, 2100, 71, alpha=True)
    a = img[..., 3]
    a[1020:1030, 10:60] = 0
    a[2040:2050, :] = 0
    compare(ctx, img, 2.0)


def test_wide_frame_with_many_holes(ctx):
    compare(ctx, synthetic.generate(2100, 300, 72, alpha=True, rectangles=20), 1.5)


def test_sixteen_bit_alpha(ctx):
    img = synthetic.generate(200, 150, 81, sixteen_bit=True, alpha=True)
    img[10:20, 10:190, 3] = 3 * 257  # fringe within REACH at 16 bits
    compare(ctx, img, 1.45)


def test_constant_alpha_keeps_the_field(ctx):
    rgb = synthetic.generate(128, 96, 91)
    half = with_alpha(rgb, np.full((96, 128), 128, np.uint8))
    got, _ = compare(ctx, half)
    plain = ctx.frontend(rgb, ultrafast(1.0))
    assert np.array_equal(got.quant_field, plain.quant_field)
    assert np.array_equal(got.tokens, plain.tokens)


def test_partial_alpha_scales_the_field(ctx):
    rgb = synthetic.generate(128, 96, 92)
    a = np.full((96, 128), 255, np.uint8)
    a[:, 64:] = 40  # a faint half: factor 40/255
    got, _ = compare(ctx, with_alpha(rgb, a))
    plain = ctx.frontend(rgb, ultrafast(1.0))
    assert np.array_equal(got.quant_field[:, :8], plain.quant_field[:, :8])
    assert np.all(got.quant_field[:, 8:] <= plain.quant_field[:, 8:])


def test_config3_rgba_frames_in_a_batch(ctx):
    imgs = [im for im in synthetic.config3_batch(8) if im.shape[2] == 4]
    cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90)
    b = ctx.batch()
    try:
        for im in imgs:
            b.add(im, cfg)
        b.run(use_graph=True)
        for i, im in enumerate(imgs):
            assert_same(b.result(i), O.frontend(im, cfg.distance), check_xyb=False)
    finally:
        b.close()


def test_bounded_wait_reports_a_timeout_and_the_context_stays_usable(ctx):
    from jixel_gb300 import _lib as L
    lib = L.load()
    assert lib.jxg_selftest_bounded_wait(ctx.handle, 2000) == 102  # JXG_ERR_DEVICE_TIMEOUT
    compare(ctx, synthetic.generate(40, 30, 99, alpha=True))
