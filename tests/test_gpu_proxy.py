"""The luma-proxy operator (jxg_op_luma_proxy) against the restatement of
the reference's scalar path (oracle/luma_proxy.py), and the reference's own
flat-field expectations (src/epf_proxy.rs:263-281)."""
import numpy as np
import pytest

import jixel_gb300 as J
from oracle import luma_proxy as P

pytestmark = pytest.mark.gpu
F = np.float32


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


@pytest.mark.parametrize("w,h,seed", [(4, 4, 1), (37, 23, 2), (257, 129, 3), (640, 360, 4)])
def test_proxy_matches_the_oracle(ctx, w, h, seed):
    # the same float32 inputs and box moments: only the pools' summation
    # order differs (the restatement's sequential float32 sums over up to
    # 460k terms drift by up to about 1e-4)
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    src = (F(0.3) + F(0.2) * np.sin(xx / 7.0 + yy / 11.0) + rng.normal(0, 0.01, (h, w))).astype(F)
    test = (src + rng.normal(0, 0.005, (h, w)).astype(F)).astype(F)
    score, terms = ctx.luma_proxy(src, test)
    want, want_terms = P.LumaProxy(src).compare(test)
    assert np.allclose(terms, want_terms.astype(np.float64), rtol=1e-4, atol=1e-7), (terms, want_terms)
    assert abs(score - float(want)) <= 1e-4 * float(want), (score, float(want))


@pytest.mark.parametrize("value", [0.0, 0.07, 0.21, 0.53, 0.91])
def test_flat_fields_keep_identity_zero(ctx, value):
    w, h = 257, 129
    y = np.full((h, w), F(value))
    identity, _ = ctx.luma_proxy(y, y)
    assert identity < 1e-5
    shifted, _ = ctx.luma_proxy(y, np.full((h, w), F(value + 0.02)))
    assert np.isfinite(shifted) and shifted > identity


def test_proxy_rejects_small_planes(ctx):
    with pytest.raises(J.EncodeError):
        ctx.luma_proxy(np.zeros((3, 8), F), np.zeros((3, 8), F))
