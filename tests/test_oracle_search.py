"""The oracle's Fastest transform search, pinned to what the reference's own
sources and tests hold (tables extracted by tests/golden/gen_golden.py)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tables.json")))

DCT, DCT16X8, DCT8X16, DCT16X16, DCT32X32 = 0, 1, 2, 3, 4
COV = {DCT: (1, 1), DCT16X8: (1, 2), DCT8X16: (2, 1), DCT16X16: (2, 2), DCT32X32: (4, 4)}


@pytest.mark.parametrize("cx,cy,key", [(1, 1, "coeff_order_8x8"), (2, 1, "coeff_order_16x8"),
                                       (2, 2, "coeff_order_16x16"), (4, 4, "coeff_order_32x32")])
def test_natural_scans_are_the_reference_tables(cx, cy, key):
    # generic_natural_scan_reproduces_the_spec_tables (src/coeff_order.rs)
    assert O.natural_scan(cx, cy).tolist() == GOLD[key]


def test_large_tables_follow_the_reference():
    t = O.large_tables(1.0)
    # dct16x8_matrix_from_bands_matches_static (src/quant_weights.rs:3392-3414):
    # the static library table is the band curve within 4e-6
    lib = np.array([float(v) for v in GOLD["dequant_matrix_16x8"]], np.float32).reshape(3, 128)
    assert np.array_equal(t["16x8"], lib)
    assert np.all(np.abs(t["16x8_bands"] - lib) <= 4e-6 * np.abs(lib))
    # dct16x16_matrix_dc_matches_libjxl_polynomial (src/quant_weights.rs:3477-3525)
    for c, b in enumerate([8996.87257, 3191.48366, 1157.50408]):
        assert abs(t["16x16"][c, 0] - 1.0 / b) < 1e-7
    assert np.all(t["16x16"] > 0) and np.all(t["16x16"][:, 255] > t["16x16"][:, 0])
    assert abs(t["32x32"][1, 0] - 1.0 / float(GOLD["dct32x32_bands"][8])) < 1e-7
    # from the SS2 gate (d >= 2.25) the 16/32 bases scale by 0.78 / 0.89
    # (QM_SS2_SCALE16 / 32, src/quant_weights.rs:115-116, :2068-2089)
    s = O.large_tables(2.5)
    assert abs(s["16x16"][1, 0] * 0.78 * 3191.48366 - 1.0) < 2e-3
    assert abs(s["32x32"][1, 0] * 0.89 * float(GOLD["dct32x32_bands"][8]) - 1.0) < 2e-3
    assert np.array_equal(s["16x8"], t["16x8"])


def _owners(m):
    yb, xb = m.shape
    owner = -np.ones((yb, xb), np.int64)
    for y in range(yb):
        for x in range(xb):
            if m[y, x] & 1:
                cx, cy = COV[int(m[y, x]) >> 1]
                assert np.all(owner[y:y + cy, x:x + cx] == -1), "cell covered twice"
                assert all((int(v) >> 1) == int(m[y, x]) >> 1 for v in m[y:y + cy, x:x + cx].ravel())
                owner[y:y + cy, x:x + cx] = y * xb + x
    assert np.all(owner >= 0), "uncovered cell"
    return owner


def test_flat_image_takes_the_32x32_and_only_squares():
    # fast_scope_selects_squares_and_no_other_merge_shape
    # (src/ac_strategy/selection.rs:4111-4150): context distance 1, search
    # distance 3, scale 1, a flat 32x32 image at field 8
    xyb = np.zeros((3, 32, 32), np.float32)
    maps = np.zeros((1, 1), np.int8)
    m, q = O.fastest_select(xyb, maps, maps, np.full((4, 4), 8, np.uint8), 1.0, 3.0, 1.0)
    assert int(m[0, 0]) == (DCT32X32 << 1) | 1
    assert all((int(v) >> 1) in (DCT, DCT16X16, DCT32X32) for v in m.ravel() if v & 1)
    assert np.all(q == 8)


def _noise_opsin(w, h, seed):
    # noise_opsin (src/ac_strategy/selection.rs:4153-4168)
    out = np.zeros((3, h, w), np.float32)
    state = seed
    for c in range(3):
        for y in range(h):
            for x in range(w):
                state = (state * 1664525 + 1013904223) & 0xFFFFFFFF
                noise = np.float32(state >> 8) / np.float32(1 << 24) - np.float32(0.5)
                out[c, y, x] = (np.float32(0.05) * noise * np.float32((y // 7) % 3)
                                + np.float32(0.002) * np.float32(y))
    return out


@pytest.mark.parametrize("distance", [2.0, 3.0, 4.5, 6.0])
def test_selector_map_is_valid_and_keeps_the_aggregated_field(distance):
    # run_selector_full's input (src/ac_strategy/selection.rs:4175-4222):
    # 13 x 11 blocks of noise over a ramp, field 4 + (3x + 5y) % 7
    bw, bh = 13, 11
    xyb = _noise_opsin(bw * 8, bh * 8, 0x9E3779B9)
    maps = np.zeros((2, 2), np.int8)
    qf = np.array([[4 + (x * 3 + y * 5) % 7 for x in range(bw)] for y in range(bh)], np.uint8)
    m, q = O.fastest_select(xyb, maps, maps, qf, distance, distance, 1.0)
    owner = _owners(m)
    # adjust_quant_field: every transform carries one field value
    for o in np.unique(owner):
        assert len(np.unique(q[owner == o])) == 1
    # no shape outside the squares scope and the re-tiling pairs
    assert all((int(v) >> 1) in COV for v in m.ravel())


def test_fastest_frontend_is_thread_invariant_and_accounts_tokens():
    # lossy_output_is_independent_of_thread_count (src/encode_image.rs:6602)
    from jixel_gb300 import synthetic
    img = synthetic.generate(300, 200, 11, rectangles=12)
    a = O.frontend(img, 2.35, num_threads=1, speed="fastest")
    b = O.frontend(img, 2.35, num_threads=4, speed="fastest")
    for k in ("quant_field", "ac_strategy", "quant_dc", "coeffs", "nzeros", "histograms"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert np.array_equal(a.tokens, b.tokens)
    assert int(a.histograms.sum()) == len(a.tokens) and a.group_offsets[-1] == len(a.tokens)
    _owners(a.ac_strategy)
    kinds = {int(v) >> 1 for v in a.ac_strategy.ravel() if v & 1}
    assert DCT16X16 in kinds or DCT32X32 in kinds
    # each multi-block transform carries one field value and one shifted count
    owner = _owners(a.ac_strategy)
    for o in np.unique(owner):
        assert len(np.unique(a.quant_field[owner == o])) == 1
        for c in range(3):
            assert len(np.unique(a.nzeros[c][owner == o])) == 1


def test_fastest_below_the_rerank_limit_is_refused_and_dct8_only_shortcut():
    from jixel_gb300 import synthetic
    img = synthetic.generate(64, 64, 3)
    with pytest.raises(ValueError):
        O.frontend(img, 1.0, speed="fastest")
    # at d <= 0.0567 the search returns at once (use_dct8_only): UltraFast's output
    a = O.frontend(img, 0.05, speed="fastest")
    b = O.frontend(img, 0.05)
    assert np.all(a.ac_strategy == 1)
    assert np.array_equal(a.tokens, b.tokens) and np.array_equal(a.quant_field, b.quant_field)


def test_all_dct8_layout_codes_like_the_dct8_path():
    # With no merge anywhere (a frame of 1x1 blocks cannot merge) the layout
    # coder reproduces the DCT8 coder bit for bit.
    from jixel_gb300 import synthetic
    img = synthetic.generate(8, 8, 5)
    a = O.frontend(img, 3.0, speed="fastest")
    b = O.frontend(img, 3.0)
    assert np.array_equal(a.tokens, b.tokens) and np.array_equal(a.quant_dc, b.quant_dc)
