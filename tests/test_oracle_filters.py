"""The oracle's Gaborish (encoder inverse and decoder forward), pinned to the
reference's own tests of them (src/gaborish.rs:260-345,
src/epf_filter/tests.rs:129-149, :255-295)."""
import numpy as np
import pytest

from oracle import oracle as O


def _ref_image(w, h):
    # image() of src/epf_filter/tests.rs:129-141
    out = np.zeros((3, h, w), np.float32)
    for c in range(3):
        for y in range(h):
            for x in range(w):
                out[c, y, x] = np.float32(0.1) + np.float32((x * 1877 + y * 6719 + c * 941) % 3253) * np.float32(0.0001)
    return out


def _mirror(i, n):
    while i < 0 or i >= n:
        i = -i - 1 if i < 0 else 2 * n - i - 1
    return i


def test_constant_input_is_unchanged_by_the_inverse():
    # constant_input_unchanged (src/gaborish.rs:319-345)
    img = np.full((3, 16, 16), 0.5, np.float32)
    out = O.gaborish_inverse(img, 0.9908511)
    assert np.all(np.abs(out - 0.5) < 1e-5)


def test_inverse_weights_are_normalised():
    w = O.gaborish_inverse_weights(0.9908511).astype(np.float64)
    assert abs(w[0] + 4 * (w[1] + w[2] + w[3] + w[5]) + 8 * w[4] - 1.0) < 1e-6
    assert w[0] > 1.0 and w[1] < 0.0  # it sharpens
    # a zero multiplier leaves the image as it is
    img = _ref_image(9, 5)
    assert np.array_equal(O.gaborish_inverse(img, 0.0), img)


@pytest.mark.parametrize("w,h", [(1, 1), (2, 3), (3, 2), (5, 7), (16, 4), (33, 17)])
def test_inverse_reflects_at_every_edge(w, h):
    # every output from source pixels with mirror-reflected neighbours, the
    # sums in the reference's order (symmetric5_row, src/gaborish.rs:136-258)
    img = _ref_image(w, h)
    k = O.gaborish_inverse_weights(0.9908511).astype(np.float64)
    got = O.gaborish_inverse(img, 0.9908511)
    for c in range(3):
        for y in range(h):
            for x in range(w):
                g = lambda dx, dy: float(img[c, _mirror(y + dy, h), _mirror(x + dx, w)])  # noqa: E731
                s_r = g(0, -1) + g(0, 1) + g(-1, 0) + g(1, 0)
                s_d = g(-1, -1) + g(1, -1) + g(-1, 1) + g(1, 1)
                s_r2 = g(0, -2) + g(0, 2) + g(-2, 0) + g(2, 0)
                s_d2 = g(-2, -2) + g(2, -2) + g(-2, 2) + g(2, 2)
                s_l = (g(-1, -2) + g(1, -2) + g(-2, -1) + g(2, -1) + g(-2, 1) + g(2, 1)
                       + g(-1, 2) + g(1, 2))
                want = (k[0] * g(0, 0) + k[1] * s_r + k[2] * s_d + k[3] * s_r2 + k[5] * s_d2
                        + k[4] * s_l)
                assert abs(got[c, y, x] - want) <= 1e-5 * max(abs(want), 1.0)


@pytest.mark.parametrize("w", list(range(1, 20)))
def test_forward_matches_the_coordinate_formula(w):
    # gaborish_matches_coordinate_oracle_without_padding
    # (src/epf_filter/tests.rs:255-295): 7 rows, widths 1..19, FMA_TOLERANCE
    img = _ref_image(w, 7)
    w0, w1, w2 = (float(v) for v in O.gaborish_weights())
    got = O.gaborish(img)
    for c in range(3):
        for y in range(7):
            for x in range(w):
                g = lambda dx, dy: float(img[c, _mirror(y + dy, 7), _mirror(x + dx, w)])  # noqa: E731
                side = (g(-1, 0) + g(1, 0)) + (g(0, -1) + g(0, 1))
                corner = (g(-1, -1) + g(1, -1)) + (g(-1, 1) + g(1, 1))
                want = corner * w2 + (side * w1 + g(0, 0) * w0)
                assert abs(got[c, y, x] - want) <= 1e-5 * max(abs(want), 1.0)


def test_forward_weights():
    w0, w1, w2 = (float(v) for v in O.gaborish_weights())
    assert abs(w0 * (1 + 4 * (w1 / w0 + w2 / w0)) - 1.0) < 1e-6
    assert abs(w1 / w0 - 1.1 * 0.10469957) < 1e-6 and abs(w2 / w0 - 1.1 * 0.05568054) < 1e-6
