"""The asynchronous front end (jxg_frontend_enqueue / jxg_frontend_wait)
returns exactly what the synchronous call returns, with the token stream
and group offsets written by the device into pinned host memory; two
contexts alternate frames as a pipelined caller would."""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic

pytestmark = pytest.mark.gpu


def same(a, b):
    assert a.params == b.params
    for k in ("quant_field", "ac_strategy", "ytox", "ytob", "quant_dc", "num_nzeros", "tokens",
              "group_offsets", "histograms"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    if a.coefficients is not None and b.coefficients is not None:
        assert np.array_equal(a.coefficients, b.coefficients)
    if a.alpha is not None and b.alpha is not None:
        assert np.array_equal(a.alpha, b.alpha)


def test_enqueue_matches_synchronous_frontend():
    torch = pytest.importorskip("torch")
    ctx = J.FrontendContext(0)
    try:
        for (w, h, kw, q) in [(640, 480, {}, 90), (300, 200, {"alpha": True}, 75),
                              (257, 65, {"sixteen_bit": True}, 95)]:
            img = synthetic.generate(w, h, 1000 + w, **kw)
            cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(q)
            want = ctx.frontend(img, cfg)
            pinned = torch.from_numpy(img.reshape(-1).view(np.uint8)).pin_memory()
            pix = pinned.numpy().view(img.dtype).reshape(img.shape)
            out = J.PinnedOutputs(w, h, channels=img.shape[2], coefficients=True)
            ctx.enqueue(pix, cfg, out)
            ctx.wait()
            same(out.result(), want)
    finally:
        ctx.close()


def test_two_contexts_pipelined():
    pytest.importorskip("torch")
    a, b = J.FrontendContext(0), J.FrontendContext(0)
    try:
        imgs = [synthetic.generate(512, 384, 2000 + i) for i in range(4)]
        cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90)
        want = [a.frontend(im, cfg) for im in imgs]
        outs = [J.PinnedOutputs(512, 384) for _ in range(2)]
        ctxs = [a, b]
        got = []
        for i, im in enumerate(imgs):
            c = ctxs[i % 2]
            if i >= 2:
                c.wait()
                got.append(outs[i % 2].result())
            c.enqueue(im, cfg, outs[i % 2])
        for i in (2, 3):
            ctxs[i % 2].wait()
            got.append(outs[i % 2].result())
        for g, w in zip(got, want):
            same(g, w)
    finally:
        a.close()
        b.close()


def test_small_token_buffer_is_reported():
    pytest.importorskip("torch")
    ctx = J.FrontendContext(0)
    try:
        img = synthetic.generate(256, 256, 77)
        out = J.PinnedOutputs(256, 256)
        out.c.token_capacity = 10
        ctx.enqueue(img, J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90), out)
        with pytest.raises(J.EncodeError):
            ctx.wait()
    finally:
        ctx.close()
