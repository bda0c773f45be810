"""apply_chroma_hf_protection on the device (jxg_op_chroma_hf_protection)
against the oracle's restatement of src/adaptive_quant.rs:222-402, bit for
bit: the reference's own stats-test image (:811-852), chromatic noise of
several shapes, a synthetic frame's XYB and adaptive field, at distances
across the fade-in and fade-out."""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic
from oracle import oracle as O
from tests.test_oracle_chroma import chromatic, reference_test_image

pytestmark = pytest.mark.gpu
DISTANCES = [0.3, 0.5, 0.75, 1.0, 1.3, 1.9, 2.5]


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def fields(xb, yb, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(1, 256, (yb, xb)).astype(np.uint8)


@pytest.mark.parametrize("w,h,amp", [(19, 17, None), (1, 1, 0.05), (7, 9, 0.05), (64, 64, 0.03),
                                     (257, 131, 0.08), (9, 200, 0.02)])
def test_chroma_hf_protection_matches_the_oracle(ctx, w, h, amp):
    xyb = reference_test_image(w, h) if amp is None else chromatic(w, h, w * h, amp)
    field = fields((w + 7) // 8, (h + 7) // 8, w + h)
    for d in DISTANCES:
        got = ctx.chroma_hf_protection(xyb, d, field)
        want = O.chroma_hf_protection(xyb, d, field)
        assert np.array_equal(got, want), (d, np.argwhere(got != want)[:4].tolist())


def test_chroma_hf_protection_on_a_frame(ctx):
    img = synthetic.generate(640, 480, 9, noise_sigma=10.0)
    res = ctx.frontend(img, J.EncodeConfig().with_quality(90), xyb=True)
    for d in (0.6, 1.0, 1.4):
        got = ctx.chroma_hf_protection(res.xyb, d, res.quant_field)
        assert np.array_equal(got, O.chroma_hf_protection(res.xyb, d, res.quant_field)), d
