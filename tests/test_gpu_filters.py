"""Gaborish on the device (jxg_op_gaborish_inverse / jxg_op_gaborish)
against the oracle, bit for bit."""
import numpy as np
import pytest

import jixel_gb300 as J
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def _planes(w, h, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.2, 1.0, (3, h, w)).astype(np.float32)


@pytest.mark.parametrize("w,h", [(1, 1), (2, 3), (3, 2), (5, 7), (33, 17), (257, 65), (1920, 1080)])
@pytest.mark.parametrize("mul", [0.9908511, 0.5])
def test_inverse_equals_the_oracle(ctx, w, h, mul):
    x = _planes(w, h, w * 7 + h)
    got = ctx.gaborish_inverse(x, mul)
    assert np.array_equal(got.view(np.uint32), O.gaborish_inverse(x, mul).view(np.uint32))


@pytest.mark.parametrize("w,h", [(1, 1), (2, 3), (19, 7), (33, 17), (257, 65), (1920, 1080)])
def test_forward_equals_the_oracle(ctx, w, h):
    x = _planes(w, h, w * 11 + h)
    got = ctx.gaborish(x)
    assert np.array_equal(got.view(np.uint32), O.gaborish(x).view(np.uint32))


def test_rejects_a_negative_multiplier(ctx):
    with pytest.raises(J.EncodeError):
        ctx.gaborish_inverse(_planes(8, 8, 1), -1.0)
