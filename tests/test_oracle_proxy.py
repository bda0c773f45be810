"""The luma-proxy restatement (oracle/luma_proxy.py) against the reference's
own tests for its box moments and its pyramid (src/epf_proxy/box_filter.rs:
491-537, src/epf_proxy.rs:251-281)."""
import numpy as np
import pytest

from oracle import luma_proxy as P

F = np.float32


def test_streamed_moments_match_the_original_box_bit_for_bit():
    # box_filter.rs:491-537: the streamed mean, square and cross moments equal
    # the full-plane box of src, src^2 and ref * src, bit for bit
    for w in list(range(1, 20)) + [31, 32, 33, 127]:
        for h in list(range(1, 10)) + [17, 65]:
            for flat in (False, True):
                i = np.arange(w * h)
                src = (np.full(w * h, F(0.21)) if flat else
                       ((i * 6719 + 941) % 65521).astype(F) * F(0.00001) - F(0.3)).reshape(h, w).astype(F)
                ref = (((i * 1877 + 11) % 3253).astype(F) * F(0.0001)).reshape(h, w).astype(F)
                mean, square = P.box_moments(src)
                assert np.array_equal(mean.view(np.uint32), P.original_box5(src).view(np.uint32)), (w, h, flat)
                assert np.array_equal(square.view(np.uint32), P.original_box5(src * src).view(np.uint32))
                m3 = P.box_moments(src, ref)
                assert np.array_equal(m3[0].view(np.uint32), mean.view(np.uint32))
                assert np.array_equal(m3[2].view(np.uint32), P.original_box5(ref * src).view(np.uint32))


def test_pyramid_halves_odd_sizes_like_separate_downsampling():
    # epf_proxy.rs:251-261: the in-place pyramid equals separate halving
    for w, h in [(2, 2), (3, 7), (16, 17), (33, 19)]:
        v = (np.arange(w * h, dtype=F) * F(0.007)).reshape(h, w)
        a = P.half(v, False)
        assert a.shape == (h // 2, w // 2)
        b = F(0.25) * (((v[0:2 * (h // 2):2, 0:2 * (w // 2):2] + v[1:2 * (h // 2):2, 0:2 * (w // 2):2]) +
                        v[0:2 * (h // 2):2, 1:2 * (w // 2):2]) + v[1:2 * (h // 2):2, 1:2 * (w // 2):2])
        assert np.array_equal(a, b.astype(F))


@pytest.mark.parametrize("value", [0.0, 0.07, 0.21, 0.53, 0.91])
def test_flat_fields_keep_identity_zero(value):
    # epf_proxy.rs:263-281 (on 257 x 129): identity below 1e-5, a shift scores higher
    w, h = 257, 129
    y = np.full((h, w), F(value))
    proxy = P.LumaProxy(y)
    identity, _ = proxy.compare(y)
    assert identity < 1e-5
    score, _ = proxy.compare(np.full((h, w), F(value + 0.02)))
    assert np.isfinite(score) and score > identity


def test_proxy_grows_with_distortion():
    rng = np.random.default_rng(7)
    y = rng.uniform(0.0, 0.6, (48, 40)).astype(F)
    proxy = P.LumaProxy(y)
    scores = [proxy.compare((y + rng.normal(0, s, y.shape)).astype(F))[0] for s in (0.0, 0.01, 0.05)]
    assert scores[0] < 1e-5 < scores[1] < scores[2]
