"""Batched passes: every frame of a batch equals the oracle's one-frame result.

A batch runs each stage as one launch over the (frame, work unit) list of
all its frames, with per-frame constants, buffers, statistics and histograms;
nothing of one frame may leak into another.  The mix covers every input
layout (RGB8, RGBA8, RGB16, RGBA16), ragged and multi-DC-group sizes, and
different distances per frame; plain and graph-replayed runs must agree.
"""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic
from oracle import oracle as O
from tests.parity import assert_same

pytestmark = pytest.mark.gpu


def ultrafast(distance):
    return J.EncodeConfig(distance=distance, speed=J.Speed.ULTRA_FAST)


MIX = [
    # (w, h, seed, kwargs, distance)
    (64, 64, 501, {}, 1.0),
    (1, 1, 502, {}, 1.0),
    (300, 200, 503, {"alpha": True}, 1.0),
    (513, 129, 504, {"sixteen_bit": True}, 1.45),
    (2100, 300, 505, {"rectangles": 30}, 2.35),
    (7, 9, 506, {"alpha": True}, 0.2783),
    (130, 70, 507, {"sixteen_bit": True, "alpha": True}, 2.0),
    (257, 65, 508, {}, 0.5),
]


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def mix():
    imgs = [synthetic.generate(w, h, seed, **kw) for (w, h, seed, kw, _) in MIX]
    wants = [O.frontend(img, d) for img, (*_, d) in zip(imgs, MIX)]
    return imgs, wants


@pytest.mark.parametrize("use_graph", [False, True])
def test_mixed_batch_matches_oracle(ctx, mix, use_graph):
    imgs, wants = mix
    b = ctx.batch()
    try:
        for img, (*_, d) in zip(imgs, MIX):
            b.add(img, ultrafast(d))
        for _ in range(2):  # the second run replays the recorded graph
            b.run(use_graph=use_graph)
            for i, want in enumerate(wants):
                assert_same(b.result(i, xyb=True), want), i
    finally:
        b.close()


def test_batch_sees_new_pixels_at_every_run(ctx):
    a = synthetic.generate(96, 80, 601)
    img = a.copy()
    b = ctx.batch()
    try:
        b.add(img, ultrafast(1.0))
        b.run(use_graph=True)
        assert_same(b.result(0), O.frontend(a, 1.0), check_xyb=False)
        img[:] = synthetic.generate(96, 80, 602)  # same buffer, new content
        b.run(use_graph=True)
        assert_same(b.result(0), O.frontend(img, 1.0), check_xyb=False)
    finally:
        b.close()


def test_batch_replans_after_another_pass(ctx):
    x = synthetic.generate(200, 150, 701)
    y = synthetic.generate(90, 300, 702)
    b = ctx.batch()
    try:
        b.add(x, ultrafast(1.0))
        b.add(y, ultrafast(1.0))
        b.run(use_graph=True)
        ctx.frontend(synthetic.generate(600, 400, 703), ultrafast(1.0))  # another pass
        with pytest.raises(J.EncodeError):
            b.result(0)  # the context now holds the other pass
        b.run(use_graph=True)  # re-planned and re-recorded
        assert_same(b.result(1), O.frontend(y, 1.0), check_xyb=False)
        b.add(synthetic.generate(33, 33, 704), ultrafast(3.0))
        b.run(use_graph=True)
        assert_same(b.result(0), O.frontend(x, 1.0), check_xyb=False)
        assert_same(b.result(2), O.frontend(synthetic.generate(33, 33, 704), 3.0),
                    check_xyb=False)
    finally:
        b.close()


def test_device_pixel_batch(ctx):
    torch = pytest.importorskip("torch")
    imgs = [synthetic.generate(160, 96, 801), synthetic.generate(75, 41, 802, sixteen_bit=True)]
    dev = [torch.from_numpy(i.view(np.uint8).reshape(-1).copy()).cuda() for i in imgs]
    torch.cuda.synchronize()
    b = ctx.batch(pixels_on_device=True)
    try:
        for img, t in zip(imgs, dev):
            h, w, ch = img.shape
            b.add_device(t.data_ptr(), w, h, ch, 16 if img.dtype == np.uint16 else 8,
                         ultrafast(1.0), keep=t)
        b.run(use_graph=True)
        for i, img in enumerate(imgs):
            assert_same(b.result(i), O.frontend(img, 1.0), check_xyb=False)
    finally:
        b.close()


def test_batch_rejects_bad_frames(ctx):
    b = ctx.batch()
    try:
        with pytest.raises(J.EncodeError) as e:
            b.add(np.zeros((0, 5, 3), np.uint8), ultrafast(1.0))
        assert e.value.variant == "EmptyImage"
        with pytest.raises(J.EncodeError) as e:
            b.add(np.zeros((8, 8, 3), np.uint8), J.EncodeConfig(distance=1.0, speed=J.Speed.FAST))
        assert e.value.variant == "Unsupported"
        with pytest.raises(J.EncodeError):
            b.run()  # nothing added
        assert len(b) == 0
    finally:
        b.close()


def test_config3_subset_matches_one_frame_passes(ctx):
    # 12 frames of the log-uniform RGB/RGBA mix: batched == one at a time
    imgs = synthetic.config3_batch(12)
    cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90)
    singles = [ctx.frontend(img, cfg) for img in imgs]
    b = ctx.batch()
    try:
        for img in imgs:
            b.add(img, cfg)
        b.run(use_graph=True)
        for i, s in enumerate(singles):
            r = b.result(i)
            for k in ("quant_field", "ytox", "ytob", "quant_dc", "coefficients", "num_nzeros",
                      "tokens", "group_offsets", "histograms"):
                assert np.array_equal(getattr(r, k), getattr(s, k)), (i, k)
            assert r.params == s.params, i
    finally:
        b.close()


def test_config3_batch_matches_the_oracle(ctx):
    # all 256 images of the log-uniform RGB/RGBA mix in one replayed batch,
    # each against the oracle's one-frame result
    imgs = synthetic.config3_batch(256)
    cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90)
    b = ctx.batch()
    try:
        for img in imgs:
            b.add(img, cfg)
        b.run(use_graph=True)
        for i, img in enumerate(imgs):
            assert_same(b.result(i), O.frontend(img, cfg.distance), check_xyb=False)
    finally:
        b.close()


def test_batch_mixes_depths_and_transfers(ctx):
    # one pass over frames of different depths and transfer functions: each
    # frame reads its own transfer table
    from tests.parity import high_depth_image
    TF = J.TransferFunction
    cases = [(synthetic.generate(90, 60, 900), 8, TF.SRGB),
             (high_depth_image(70, 50, 901, 10), 10, TF.SRGB),
             (high_depth_image(64, 64, 902, 16), 16, TF.LINEAR),
             (high_depth_image(50, 70, 903, 12, alpha=True), 12, TF.BT709),
             (synthetic.generate(40, 30, 904), 8, TF.BT709)]
    b = ctx.batch()
    try:
        for img, bits, tf in cases:
            b.add(img, J.EncodeConfig(distance=1.0, speed=J.Speed.ULTRA_FAST, transfer=tf,
                                      bits_per_sample=bits))
        b.run()
        for i, (img, bits, tf) in enumerate(cases):
            assert_same(b.result(i), O.frontend(img, 1.0, bits=bits, transfer=int(tf)),
                        check_xyb=False)
    finally:
        b.close()
