"""The decoder's EPF operator (jxg_op_epf) against the restatement of the
reference's own coordinate oracle (oracle/epf.py), bit for bit, on the
inputs of the reference's test (src/epf_filter/tests.rs:168-222): its image
generator, the mixed block sigmas and the seven loop-filter candidates, over
every size of its list."""
import numpy as np
import pytest

import jixel_gb300 as J
from oracle import epf as E

pytestmark = pytest.mark.gpu
F = np.float32

SIZES = [(w, 19 - w) for w in range(1, 18)] + [(35, 27), (65, 49), (130, 11)]
# (iters, quant_mul, sharpness, pass0), each LoopFilter::new(iters, Some(pass0),
# Some(q), Some([31, 6, 4.5])): the bundle through F16
CANDIDATES = [(3, 0.46, 7, 0.9), (1, 1.84, 3, 0.9), (2, 0.46, 7, 0.9), (3, 1.84, 7, 3.6),
              (2, 0.12, 7, 0.9), (0, 0.46, 7, 0.9), (1, 0.46, 0, 0.9)]


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def image(w, h):
    x, y = np.arange(w), np.arange(h)
    return np.stack([(F(0.1) + ((x[None, :] * 1877 + y[:, None] * 6719 + c * 941) % 3253).astype(F) * F(0.0001))
                     .astype(F) for c in range(3)])


@pytest.mark.parametrize("w,h", SIZES)
def test_epf_matches_the_reference_oracle_bit_for_bit(ctx, w, h):
    img = image(w, h)
    nb = ((w + 7) // 8) * ((h + 7) // 8)
    sq = np.array([[-0.1, -1.0, -10.0, 0.0][i % 4] for i in range(nb)], F)
    cs = [E.f16(31.0), E.f16(6.0), E.f16(4.5)]
    for iters, q, sharp, pass0 in CANDIDATES:
        args = (iters, E.f16(q), E.f16(pass0), E.f16(6.5), E.f16(2.0 / 3.0), cs, sharp)
        want = E.epf(img, sq, *args)
        got = ctx.epf(img, sq, iters, float(args[1]), float(args[2]), float(args[3]), float(args[4]),
                      [float(v) for v in cs], sharp)
        bad = np.argwhere(got.view(np.uint32) != want.view(np.uint32))
        assert bad.size == 0, (iters, q, sharp, pass0, bad[:4].tolist(),
                               got[tuple(bad[0])] if bad.size else None, want[tuple(bad[0])] if bad.size else None)


def test_epf_rejects_bad_arguments(ctx):
    img = image(16, 16)
    sq = np.full(4, -1.0, F)
    with pytest.raises(J.EncodeError):
        ctx.epf(img, sq, 4)
    with pytest.raises(J.EncodeError):
        ctx.epf(img, np.full(3, -1.0, F), 1)
