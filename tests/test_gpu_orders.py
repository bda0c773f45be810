"""The order-statistics kernel (jxg_order_stats) against the restatement of
OrderStats::tally (oracle/coeff_order.py) over the oracle's own pass-one
levels and strategy map, bit for bit, on UltraFast and Speed::Fastest frames;
then the orders derived from the device's statistics against the
restatement's."""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic
from oracle import coeff_order as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


CASES = [
    # (width, height, seed, quality, speed): all-DCT8 frames, then searched
    # layouts with 16x8 / 8x16 / 16x16 / 32x32 pieces
    (512, 512, 1, 90, "ultrafast"),
    (1000, 700, 2, 75, "ultrafast"),
    (1024, 768, 3, 75, "fastest"),
    (1920, 1080, 4, 60, "fastest"),
]


@pytest.mark.parametrize("w,h,seed,q,speed", CASES)
def test_order_stats_match_the_oracle(ctx, w, h, seed, q, speed):
    img = synthetic.generate(w, h, seed)
    cfg = J.EncodeConfig(speed=J.Speed.FASTEST if speed == "fastest" else J.Speed.ULTRA_FAST).with_quality(q)
    res = ctx.frontend(img, cfg)
    counts, blocks = ctx.order_stats()
    want = O.frontend(img, J.distance_from_quality(q), speed=speed)
    assert np.array_equal(res.ac_strategy, want.ac_strategy)
    want_counts, want_blocks = C.tally(want.coeffs, want.ac_strategy if speed == "fastest" else None)
    assert blocks.tolist() == want_blocks
    for slot in range(len(C.ORDER_SPECS)):
        assert np.array_equal(counts[slot], want_counts[slot]), slot
    if speed == "fastest":
        assert sum(blocks[s] > 0 for s in (0, 2, 3, 4)) >= 3  # the searched layout mixes shapes
    used, orders, moved = J.derive_orders(counts, blocks)
    want_used, want_orders, want_moved = C.derive_orders(want_counts, want_blocks)
    assert used == want_used and moved == want_moved
    for slot in range(len(C.ORDER_SPECS)):
        assert np.array_equal(orders[slot], np.array(want_orders[slot], np.uint32)), slot


def test_order_stats_need_a_pass():
    c = J.FrontendContext(0)
    try:
        with pytest.raises(J.EncodeError):
            c.order_stats()
    finally:
        c.close()
