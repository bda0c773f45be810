"""Parity of the Speed::Fastest front end with the oracle (bit-exact): the
transform search (strategy map and adjusted quant field), then the coding of
the layout (DC and AC levels, non-zero counts, tokens, histograms)."""
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


def fastest(distance, bits=0, transfer=J.TransferFunction.SRGB):
    return J.EncodeConfig(distance=distance, speed=J.Speed.FASTEST, bits_per_sample=bits,
                          transfer=transfer)


def compare(ctx, img, distance, bits=0, transfer=J.TransferFunction.SRGB):
    want = O.frontend(img, distance, bits=bits or None, transfer=int(transfer), speed="fastest")
    got = ctx.frontend(img, fastest(distance, bits, transfer), xyb=False)
    # the search first: a different layout changes everything after it
    if not np.array_equal(got.ac_strategy, want.ac_strategy):
        bad = np.argwhere(got.ac_strategy != want.ac_strategy)
        raise AssertionError(f"strategy map differs at {len(bad)} blocks, first {bad[:4].tolist()}")
    assert np.array_equal(got.quant_field, want.quant_field), "adjusted quant field"
    assert_same(got, want, check_xyb=False)
    return got, want


@pytest.mark.parametrize("q", [80, 75, 60, 40, 20, 5])
def test_config1_qualities(ctx, q):
    got, _ = compare(ctx, synthetic.config1_image(), J.distance_from_quality(q))
    kinds = {int(v) >> 1 for v in got.ac_strategy.ravel() if v & 1}
    assert kinds & {3, 4}, "no merge placed"


@pytest.mark.parametrize("w,h", [(1, 1), (9, 7), (24, 40), (33, 33), (65, 65), (130, 66),
                                 (257, 129), (300, 97)])
def test_ragged_sizes(ctx, w, h):
    compare(ctx, synthetic.generate(w, h, 5 + w * h, rectangles=4), 2.5)


def test_between_the_rerank_limit_and_the_ss2_gate(ctx):
    # 1.709 < d < 2.25: library 16x16 / 32x32 tables, no matrix-header pass
    compare(ctx, synthetic.config1_image(), 1.9)


def test_two_dc_groups_and_edges(ctx):
    img = synthetic.generate(2100, 300, 21, noise_sigma=4.0, rectangles=40, texture_weight=0.3)
    compare(ctx, img, 2.35)


def test_rgba_alpha_factors_follow_the_layout(ctx):
    img = synthetic.generate(320, 200, 31, alpha=True)
    compare(ctx, img, 2.2)
    compare(ctx, img, 3.0)


def test_sixteen_bit_and_grey(ctx):
    img16 = synthetic.generate(200, 136, 41, sixteen_bit=True)
    compare(ctx, img16, 2.6, bits=16, transfer=J.TransferFunction.LINEAR)
    grey = synthetic.generate(180, 120, 43)[..., 1]
    compare(ctx, grey, 2.4)


def test_flat_screen_content(ctx):
    img = np.full((256, 256, 3), 200, np.uint8)
    img[64:192, 64:192] = (10, 90, 220)
    got, _ = compare(ctx, img, 3.0)
    assert got.params["screen_content"]


def test_reranked_distances_are_refused_and_the_dct8_shortcut_is_ultrafast(ctx):
    img = synthetic.generate(64, 48, 7)
    with pytest.raises(J.EncodeError) as e:
        ctx.frontend(img, fastest(1.0))
    assert e.value.variant == "Unsupported"
    a = ctx.frontend(img, fastest(0.05), xyb=False)
    b = ctx.frontend(img, J.EncodeConfig(distance=0.05, speed=J.Speed.ULTRA_FAST), xyb=False)
    assert np.all(a.ac_strategy == 1) and np.array_equal(a.tokens, b.tokens)


def test_config2_frame_at_q75_whole(ctx):
    # the benchmarked 3840x2160 frame at q75, compared whole
    compare(ctx, synthetic.config2_image(), J.distance_from_quality(75))


def test_serial_sums_give_the_same_frame(ctx, monkeypatch):
    # JXG_SERIAL_SUMS=1 takes every f64 running sum serially in the
    # reference's order instead of settling it from a parallel sum's interval
    monkeypatch.setenv("JXG_SERIAL_SUMS", "1")
    compare(ctx, synthetic.config1_image(), J.distance_from_quality(40))
    compare(ctx, synthetic.generate(2100, 300, 21, noise_sigma=4.0, rectangles=40,
                                    texture_weight=0.3), 2.35)


def test_black_regions_take_the_serial_variance(ctx):
    # black luma sits below 2^-19, where the site variance's exact integer
    # sum does not apply and the serial f64 sums run
    img = synthetic.generate(256, 192, 51, rectangles=10)
    img[32:160, 40:200] = 0
    img[100:120, 0:256] = (3, 2, 1)
    compare(ctx, img, 2.6)


def test_launch_geometry_does_not_change_the_frame(ctx):
    # warps per CTA of the tunable kernels: every choice codes the same frame
    img = synthetic.config1_image()
    d = J.distance_from_quality(60)
    want = O.frontend(img, d, speed="fastest")
    base = ctx.launch_geometry()
    try:
        for w in (1, 2, 8):
            ctx.set_launch_geometry({k: w for k in base})
            got = ctx.frontend(img, fastest(d), xyb=False)
            assert np.array_equal(got.ac_strategy, want.ac_strategy), w
            assert_same(got, want, check_xyb=False)
        with pytest.raises(J.EncodeError):
            ctx.set_launch_geometry({"k_retile": 3})
    finally:
        ctx.set_launch_geometry(base)


def test_autotune_picks_a_geometry_that_codes_the_same_frame(ctx):
    torch = pytest.importorskip("torch")
    img = synthetic.config1_image()
    d_img = torch.from_numpy(img).cuda().contiguous()
    base = ctx.launch_geometry()
    try:
        geo, times = ctx.autotune(d_img.data_ptr(), img.shape[1], img.shape[0], 3, 8,
                                  fastest(J.distance_from_quality(75)), rounds=1)
        assert set(geo.values()) <= {1, 2, 4, 8}
        for k, t in times.items():
            assert all(np.isfinite(v) and v > 0 for v in t.values()), k
            assert t[geo[k]] == min(t.values()), k
        compare(ctx, img, J.distance_from_quality(75))
    finally:
        ctx.set_launch_geometry(base)
