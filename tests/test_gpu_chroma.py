"""pixel_chromacity_steps on the device (jxg_pixel_chromacity, over the last
pass's XYB) against the oracle's restatement of src/frame/chroma.rs:89-165 on
the same planes, bit for bit: frames of several shapes, colour and grey."""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


@pytest.mark.parametrize("w,h,seed,grey", [(1, 1, 1, False), (2, 2, 2, False), (1, 40, 3, False),
                                           (33, 1, 4, False), (257, 131, 5, False),
                                           (1920, 1080, 6, False), (640, 480, 7, True)])
def test_pixel_chromacity_matches_the_oracle(ctx, w, h, seed, grey):
    img = synthetic.generate(w, h, seed, noise_sigma=12.0)
    if grey:
        img = img[:, :, 1].copy()
    res = ctx.frontend(img, J.EncodeConfig().with_quality(75), xyb=True)
    counts, xs, bs = ctx.pixel_chromacity()
    want, wx, wb = O.pixel_chromacity(res.xyb)
    assert np.array_equal(counts, want), (counts, want)
    assert (xs, bs) == (wx, wb)
