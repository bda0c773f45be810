"""The restatement of pixel_chromacity_steps (oracle orc_pixel_chromacity,
src/frame/chroma.rs:89-165) against a second, vectorised statement of the same
formula (the left and upper neighbours of every pixel past the first row and
column), on random and structured planes of every small shape.  The reference
has no test of its own for this function; its formula is read from
src/frame/chroma.rs:100-165."""
import numpy as np
import pytest

from oracle import oracle as O

F = np.float32


def vectorised(xyb):
    X, Y, B = (xyb[c].astype(F) for c in range(3))
    h, w = X.shape
    if w < 2 or h < 2:
        return np.zeros(7, np.uint32), 0, 0
    x, y, b = X[1:, 1:], Y[1:, 1:], B[1:, 1:]
    lx, lb, ly = X[1:, :-1], B[1:, :-1], Y[1:, :-1]
    px, pb, py = X[:-1, 1:], B[:-1, 1:], Y[:-1, 1:]
    step_x = np.maximum(np.abs(x - lx), np.abs(x - px))
    diff = (b - y).astype(F)
    step_b = np.maximum(np.abs(diff - (lb - ly).astype(F)), np.abs(diff - (pb - py).astype(F)))
    step = (np.abs(b - lb) + np.abs(b - pb)).astype(F)
    exposed = ((b - (y * F(1.2)).astype(F)).astype(F) * step).astype(F) >= F(0.13)
    counts = [np.count_nonzero(step_x >= F(v)) for v in (0.015, 0.022, 0.026)]
    counts += [np.count_nonzero(step_b > F(v)) for v in (0.28, 0.33, 0.38)]
    counts.append(np.count_nonzero(exposed))
    lx_ = sum(c >= 4 for c in counts[:3])
    lb_ = sum(c >= 4 for c in counts[3:6])
    return np.array(counts, np.uint32), lx_, (0 if lb_ == 0 else lb_ - 1 + (counts[6] > 0))


@pytest.mark.parametrize("w,h", [(1, 1), (1, 9), (9, 1), (2, 2), (3, 17), (17, 3), (64, 48), (257, 31)])
@pytest.mark.parametrize("scale", [0.01, 0.2, 1.0])
def test_restatement_matches_the_formula(w, h, scale):
    rng = np.random.default_rng(w * 1000 + h)
    xyb = (rng.normal(0, scale, (3, h, w)) + np.array([0.0, 0.4, 0.45])[:, None, None]).astype(F)
    counts, xs, bs = O.pixel_chromacity(xyb)
    want, wx, wb = vectorised(xyb)
    assert np.array_equal(counts, want) and (xs, bs) == (wx, wb)


def test_flat_and_grey_planes_take_no_steps():
    xyb = np.zeros((3, 40, 40), F)
    xyb[1] = xyb[2] = 0.3
    assert O.pixel_chromacity(xyb)[1:] == (0, 0)
    # a snapped grey frame (X = 0, B = Y) with luma texture: no X or B - Y steps
    rng = np.random.default_rng(3)
    xyb[1] = rng.uniform(0, 0.8, (40, 40)).astype(F)
    xyb[2] = xyb[1]
    counts, xs, bs = O.pixel_chromacity(xyb)
    assert counts[:6].sum() == 0 and xs == 0 and bs == 0


def reference_test_image(w=19, h=17):
    """The image of selected_chroma_hf_stats_match_scalar (src/adaptive_quant.rs:811-852)."""
    y, x = np.mgrid[0:h, 0:w]
    return np.stack([((((x * 37 + y * 53 + c * 97 + x * y * 3) % 257).astype(F) - F(128)) / F(211))
                     .astype(F) for c in range(3)])


def chromatic(w, h, seed, amp):
    rng = np.random.default_rng(seed)
    xyb = np.zeros((3, h, w), F)
    xyb[1] = 0.4 + rng.normal(0, 0.002, (h, w))
    xyb[0] = amp * np.sign(rng.normal(0, 1, (h, w)))
    xyb[2] = xyb[1] + amp * 4 * np.sign(rng.normal(0, 1, (h, w)))
    return xyb.astype(F)


def test_chroma_hf_protection_only_raises_in_its_distance_band():
    # ChromaHfFit (src/adaptive_quant.rs:319-342): fades in from 0.35, out at 2
    xyb = chromatic(40, 24, 1, 0.05)
    field = np.full((3, 5), 40, np.uint8)
    for d in (0.2, 0.35, 2.0, 3.0):
        assert np.array_equal(O.chroma_hf_protection(xyb, d, field), field), d
    for d in (0.5, 0.75, 1.0, 1.5):
        out = O.chroma_hf_protection(xyb, d, field)
        assert np.all(out >= field) and np.any(out > field), d
        assert np.all(out <= np.round(field * (1.0 + 1.75 * 0.4)) + 1)


def test_chroma_hf_protection_leaves_achromatic_blocks():
    xyb = reference_test_image()
    xyb[0] = 0.0
    xyb[2] = xyb[1]
    field = np.arange(9, dtype=np.uint8).reshape(3, 3) * 20 + 5
    assert np.array_equal(O.chroma_hf_protection(xyb, 0.9, field), field)
