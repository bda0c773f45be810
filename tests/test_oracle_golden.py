"""Pin the CPU oracle against the reference's own known answers.

The reference ships no golden images; what it pins are constant tables and
asserted values in its unit tests (extracted by tests/golden/gen_golden.py).
"""
import json
import math
import os
import struct

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tables.json")))


def f32_bits(v):
    return struct.unpack("<I", struct.pack("<f", v))[0]


def test_natural_scan_matches_reference_table():
    assert O.natural_scan_8x8().tolist() == GOLD["coeff_order_8x8"]


def test_zero_density_context_tables():
    lib = O.lib()
    for k in range(1, 64):
        assert lib.orc_freq_context(k) == GOLD["coeff_freq_context"][k]
        assert lib.orc_nonzero_context(k) == GOLD["coeff_num_nonzero_context"][k]


def test_exp2_table_matches_reference():
    import ctypes
    t = np.zeros(64, np.float32)
    O.lib().orc_exp2_table(t.ctypes.data_as(ctypes.c_void_p))
    assert [f32_bits(float(v)) for v in t] == GOLD["exp2_table_hi_bits"]


def test_quality_anchor_points():
    tol = GOLD["quality_anchor_tolerance"]
    for q, d in GOLD["quality_anchors"]:
        assert abs(O.distance_from_quality(q) - d) < tol, (q, d)
    lo, hi = GOLD["quality_25_range"]
    assert lo < O.distance_from_quality(25.0) < hi


def test_hybrid_uint_and_pack_signed():
    lib = O.lib()
    for v, tok in GOLD["hybrid_uint"]:
        assert lib.orc_hybrid_token(v) == tok
    assert lib.orc_hybrid_token(0xFFFFFFFF) == 127


def test_dirty_log2f_exact_on_powers_of_two():
    lo, hi = GOLD["dirty_log2f_pow2_exponents"]
    for e in range(lo, hi + 1):
        assert O.lib().orc_dirty_log2f(2.0 ** e) == float(e)


def test_dirty_log2f_accuracy():
    # src/adaptive_quant.rs:903-916: max abs error < 2e-6 over [1e-6, 1e6]
    x = 1.0e-6
    worst = 0.0
    while x <= 1.0e6:
        xf = np.float32(x)
        worst = max(worst, abs(O.lib().orc_dirty_log2f(float(xf)) - math.log2(float(xf))))
        x *= 1.01
    assert worst < 2.0e-6


def test_dc_steps_are_f16_exact():
    # src/frame/quantization.rs:246-275: signalled DC steps survive the wire
    for d in [1.4, 2.0, 4.5, 6.0, 11.0, 25.0]:
        p = O.params(d)
        for c, s in enumerate(p["dc_step"]):
            dq = [1 / 4096, 1 / 512, 1 / 256][c]
            wire = np.float32(np.float32(dq) * np.float32(128.0) * np.float32(s))
            assert np.float32(np.float16(wire)) == wire


def test_params_known_values_q90():
    p = O.params(O.distance_from_quality(90))
    assert p["global_scale"] == 5243
    assert p["x_qm_scale"] == 2 and p["epf_iters"] == 1
    assert p["dc_step"] == [2.0, 1.0, 1.0]


def test_epf_sharpness_schedule():
    lib = O.lib()
    assert lib.orc_epf_sharpness_id(1.0, 0) == 7
    assert lib.orc_epf_sharpness_id(1.5, 0) == 6
    assert lib.orc_epf_sharpness_id(2.0, 1) == 7
    assert lib.orc_epf_sharpness_id(2.0, 0) == 5
    assert lib.orc_epf_sharpness_id(4.0, 0) == 4
    assert lib.orc_epf_sharpness_id(25.0, 0) == 1


def test_constant_block_fraction_reference_case():
    # src/frame/chroma.rs:496-511: left half flat, right half ramp -> 4 of 8
    xyb = np.zeros((3, 16, 32), np.float32)
    xyb[:, :, 16:] = (np.arange(16, 32, dtype=np.float32) * 0.01)[None, None, :]
    n = O.lib().orc_constant_blocks(xyb.ctypes.data, 32, 16)
    assert n == 4
    assert O.lib().orc_constant_blocks(np.zeros((3, 7, 7), np.float32).ctypes.data, 7, 7) == 0


def test_dct8_round_trip_against_float64():
    # forward DCT8 (scaled 1/64, transposed storage) vs an exact float64 DCT-II
    rng = np.random.default_rng(5)
    blk = rng.uniform(-1, 1, (8, 8)).astype(np.float32)
    got = O.dct8x8(blk).reshape(8, 8)
    n = np.arange(8)
    c = np.cos(np.pi * (2 * n[None, :] + 1) * n[:, None] / 16)
    scale = np.where(n == 0, 1 / 8, 1 / (8 * np.sqrt(2)) * 2 / np.sqrt(2) * np.sqrt(2) / 2)
    # reference scaling: DC = mean, AC = 2/N-normalised with sqrt(2) gain
    ref = c @ blk.astype(np.float64) @ c.T
    dc_expected = blk.astype(np.float64).mean()
    assert abs(got[0, 0] - dc_expected) < 1e-6
    # coefficient (u, v) lands at [v][u]: transposed storage
    ratio = got[1:, 0] / (ref[0, 1:] / 64.0)
    assert np.allclose(ratio, ratio[0], rtol=1e-4)


def test_frontend_token_accounting():
    img = np.random.default_rng(7).integers(0, 256, (40, 72, 3), dtype=np.uint8)
    f = O.frontend(img, 1.0)
    # every block-channel emits its non-zero count token; histogram counts every token
    xb, yb = 9, 5
    assert int(f.histograms.sum()) == len(f.tokens)
    assert len(f.tokens) >= 3 * xb * yb
    assert f.group_offsets[-1] == len(f.tokens)
    # the quantized coefficients' non-zero counts equal the stored counts
    nz = (f.coeffs[..., 1:] != 0).sum(-1)  # (yb, xb, 3)
    assert np.array_equal(nz.transpose(2, 0, 1), f.nzeros)


def test_low_distance_uses_library_table():
    m, inv = O.dct8_tables(0.2)
    # spec DCT8 X/Y/B base weights: 1/3150, 1/560, 1/512 at the DC position
    assert abs(m[0, 0] - 1 / 3150) < 1e-9 and abs(m[1, 0] - 1 / 560) < 1e-8
    assert abs(m[2, 0] - 1 / 512) < 1e-8
    assert np.all(inv[:, 0] == 0) and np.allclose(inv[:, 1:] * m[:, 1:], 1, rtol=1e-6)


# --- alpha: the reference's own known-answer tests, restated on the oracle ---

def test_alpha_fringe_clears_thin_edges_and_keeps_shadow_tails():
    # src/alpha_fringe.rs:233-262
    w, h = 64, 64
    a = np.zeros((h, w), np.uint16)
    a[:, 0:20] = 255
    a[:, 20] = 3
    a[20:51, 40:64] = 2
    got = O.alpha_fringe_clear(a, 255)
    assert np.all(got[:, 20] == 0)
    assert got[35, 52] == 2
    assert got[35, 10] == 255
    deep = O.alpha_fringe_clear(a.astype(np.uint32) * 257, 65535)
    assert np.array_equal(deep, got.astype(np.uint32) * 257)


def test_alpha_fringe_fills_dithered_backdrop_only_when_broad():
    # src/alpha_fringe.rs:264-299
    w, h = 64, 64
    y, x = np.mgrid[0:h, 0:w]
    a = np.where(y <= 7, 128, np.where((x + 2 * y) % 4 == 0, 254, 255)).astype(np.uint16)
    got = O.alpha_fringe_clear(a, 255)
    assert np.all(got[8:] == 255)
    assert np.all(got[:8] == 128)
    deep = O.alpha_fringe_clear(a.astype(np.uint32) * 257, 65535)
    assert np.array_equal(deep, got.astype(np.uint32) * 257)
    sparse = np.full(w * h, 255, np.uint16)
    sparse[::40] = 254
    sparse = sparse.reshape(h, w)
    assert np.array_equal(O.alpha_fringe_clear(sparse, 255), sparse)
    shade = np.full((h, w), 253, np.uint16)
    assert np.array_equal(O.alpha_fringe_clear(shade, 255), shade)


def _planes(w, h, values):
    return np.stack([np.array(values, np.float32).reshape(h, w)] * 3)


def test_fill_invisible_propagates_in_scan_order():
    # src/invisible.rs:158-175
    img = _planes(3, 2, [2.0, 99.0, 4.0, 6.0, 99.0, 99.0])
    got = O.fill_invisible(img, np.array([[255, 0, 1], [128, 0, 0]], np.uint16))
    want = np.array([2.0, 3.0, 4.0, 6.0, 4.8, 4.266667], np.float32)
    for c in range(3):
        assert np.allclose(got[c].reshape(-1), want, atol=1e-6)


def test_fill_invisible_rows_columns_and_fully_transparent():
    # src/invisible.rs:177-195 (the non-empty cases)
    for w, h, alpha, src, want in [
        (1, 1, [0], [99.0], [0.0]),
        (3, 1, [0, 1, 0], [99.0, 2.0, 99.0], [2.0] * 3),
        (1, 3, [0, 1, 0], [99.0, 2.0, 99.0], [2.0] * 3),
        (2, 2, [0] * 4, [99.0] * 4, [0.0] * 4),
    ]:
        got = O.fill_invisible(_planes(w, h, src), np.array(alpha, np.uint16).reshape(h, w))
        for c in range(3):
            assert got[c].reshape(-1).tolist() == want


def test_fill_invisible_high_depth_uses_opacity():
    # src/invisible.rs:223-239: 16-bit alpha gives the 8-bit result
    ref = O.fill_invisible(_planes(3, 1, [99.0, 2.0, 99.0]), np.array([[0, 1, 0]], np.uint16))
    deep = O.fill_invisible(_planes(3, 1, [99.0, 2.0, 99.0]), np.array([[0, 1, 0]], np.uint16))
    assert np.array_equal(ref, deep)


def test_alpha_factors_follow_each_blocks_largest_alpha():
    # src/adaptive_quant.rs:1077-1099
    w, h = 24, 8
    a = np.zeros((h, w), np.uint16)
    a[:, 8:24] = 10
    a[3, 12] = 255
    f = O.alpha_block_factors(a, 255)
    assert f.shape == (1, 3)
    assert f[0, 0] == 1.0 and f[0, 1] == 1.0
    assert abs(f[0, 2] - 0.1) < 1e-6
    a[3, 12] = 128
    assert abs(O.alpha_block_factors(a, 255)[0, 1] - 128.0 / 255.0) < 1e-6


def test_dct8_bands_and_matrix_match_the_static_table():
    # src/quant_weights.rs:3367-3390: the band parameters reproduce the
    # static DCT8 table within 2e-6 relative
    bands = np.array(GOLD["dct8_bands"], np.float32).reshape(3, 6)
    assert np.array_equal(O.dct8_default_bands(), bands)
    got = O.dct8_matrix_from_bands(bands)
    want = np.array(GOLD["dequant_matrix_8x8"], np.float32).reshape(3, 64)
    assert np.all(np.abs(got - want) <= 2e-6 * np.abs(want))


def test_fast_tables_flat_b_row_above_the_ss2_distance():
    # src/quant_weights.rs:3350-3364: new_fast's B row starts at 512 from d = 2.25;
    # its DC weight is 1 / 512 in the decoded table
    for d in [2.25, 3.0, 3.5, 5.0]:
        m, _ = O.dct8_tables(d)
        assert m[2][0] == np.float32(1.0) / np.float32(512.0)


def test_oracle_is_thread_invariant():
    # src/encode_image.rs:6602 (thread invariance): the fan-out over DC
    # groups, tiles and AC groups does not change any output
    from jixel_gb300 import synthetic
    img = synthetic.generate(600, 300, 77, rectangles=10, alpha=True)
    a = O.frontend(img, 1.0, num_threads=1)
    b = O.frontend(img, 1.0, num_threads=4)
    for k in ("quant_field", "ytox", "ytob", "quant_dc", "coeffs", "nzeros", "tokens",
              "group_offsets", "histograms", "alpha"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert np.array_equal(a.xyb.view(np.uint32), b.xyb.view(np.uint32))


def test_cfl_perfectly_correlated_chroma_finds_the_slope():
    # src/color_correlation.rs:2335-2357: X = 0.3 Y gives ytox ~ 25, B = Y ytob ~ 0
    y, x = np.mgrid[0:64, 0:64]
    v = ((x ^ y).astype(np.float32) / np.float32(64.0)).astype(np.float32)
    xyb = np.stack([np.float32(0.3) * v, v, v]).astype(np.float32)
    ytox, ytob = O.cmap_tile0(xyb, 2.0)
    assert abs(ytox - 25) < 3, ytox
    assert abs(ytob) < 3, ytob


def test_srgb_lut_is_the_reference_formula():
    # src/color.rs:35-42 (lut_matches_reference :628): f64 sRGB EOTF of v / 255
    # (v * (1 / 255.0)), rounded once to f32
    v = np.arange(256, dtype=np.float64) * (1.0 / 255.0)
    want = np.where(v <= 0.04045, v / 12.92, ((v + 0.055) / 1.055) ** 2.4).astype(np.float32)
    assert np.array_equal(O.srgb_lut().view(np.uint32), want.view(np.uint32))


def _pairs(words, woffs, goffs):
    from jixel_gb300.api import unpack_tokens
    return unpack_tokens(words, woffs, goffs).tolist()


def test_packed_token_boundaries_and_wide_fallback():
    # src/entropy/token_stream.rs:250-277: the largest context and value still
    # pack (one word each); one value or context past them, or u32::MAX, keeps
    # the whole stream wide; both forms give back every bit
    mc, mv = O.PACKED_MAX_CONTEXT, O.PACKED_MAX_VALUE
    assert (mc, mv) == ((1 << 14) - 1, (1 << 18) - 1)
    assert O.NUM_FINE_AC_CONTEXTS - 1 <= mc
    source = [[0, 0], [mc, mv], [O.NUM_FINE_AC_CONTEXTS - 1, 31]]
    words, woffs = O.ac_tokens_from(np.array(source), np.array([0, 3]))
    assert woffs.tolist() == [0, 3] and words.dtype == np.uint32
    assert [O.ac_token_unpack(int(w)) for w in words] == [tuple(t) for t in source]
    for wide in ([0, mv + 1], [mc + 1, 0], [0xFFFFFFFF, 0xFFFFFFFF]):
        src = source + [wide]
        words, woffs = O.ac_tokens_from(np.array(src, np.uint64).astype(np.uint32), np.array([0, 4]))
        assert woffs.tolist() == [0, 8]
        assert _pairs(words, woffs, np.array([0, 4], np.uint64)) == src


def test_packed_token_views_and_empty_streams():
    # src/entropy/token_stream.rs:279-310: 97 tokens (i % 7, 13 i), with and
    # without a u32::MAX value at the end; an empty stream packs to nothing
    for wide in (False, True):
        src = np.array([[i % 7, 0xFFFFFFFF if wide and i == 96 else 13 * i] for i in range(97)],
                       np.uint64).astype(np.uint32)
        words, woffs = O.ac_tokens_from(src, np.array([0, 97]))
        assert int(woffs[-1]) == (194 if wide else 97)
        assert np.array_equal(np.array(_pairs(words, woffs, np.array([0, 97], np.uint64))), src)
    words, woffs = O.ac_tokens_from(np.zeros((0, 2), np.uint32), np.array([0, 0]))
    assert words.size == 0 and woffs.tolist() == [0, 0]


def test_packed_form_is_decided_per_group():
    # AcTokens::from runs on each group's own stream (src/frame/ac_groups.rs:243):
    # a wide group leaves its neighbours packed; offsets need not start at 0
    toks = np.array([[1, 2], [3, 4], [5, 1 << 18], [6, 7], [8, 9]], np.uint32)
    goffs = np.array([10, 12, 13, 13, 15], np.uint64)
    words, woffs = O.ac_tokens_from(toks, goffs)
    assert woffs.tolist() == [0, 2, 4, 4, 6]
    assert words[:2].tolist() == [(1 << 18) | 2, (3 << 18) | 4]
    assert words[2:4].tolist() == [5, 1 << 18]
    assert _pairs(words, woffs, goffs) == toks.tolist()


@pytest.mark.parametrize("n", [32, 64, 128])
def test_dct1d_diagonalizes_the_dct_basis(n):
    # src/dct.rs:3265-3289 (32 points; the 64-point recursion alike): the
    # k0-th DCT-II basis vector peaks at k0 only
    for k0 in range(n):
        x = np.array([math.cos(np.float32(math.pi) * (2.0 * i + 1.0) * k0 / (2.0 * n))
                      for i in range(n)], np.float32)
        y = O.dct1d(x)
        mi = int(np.argmax(np.abs(y)))
        mv = float(abs(y[mi]))
        assert mi == k0, (k0, mi)
        off = float(sum(float(y[i]) ** 2 for i in range(n) if i != k0))
        assert off < 1e-6 * max(mv * mv, 1.0), (k0, off)


def _lcg_block(count):
    # the reference test's generator (src/dct.rs:3305-3310)
    rng, out = 0x9E3779B9, []
    for _ in range(count):
        rng = (rng * 1664525 + 1013904223) & 0xFFFFFFFF
        out.append(np.float32(rng >> 8) / np.float32(1 << 24) - np.float32(0.5))
    return np.array(out, np.float32)


@pytest.mark.parametrize("name,n", [("32x32", 32), ("16x16", 16)])
def test_square_dct_matches_separable_reference(name, n):
    # src/dct.rs:3291-3337: the 2-D transform equals columns then rows of the
    # probed 1-D kernel, scaled 1/n^2, stored transposed
    m1 = np.zeros((n, n), np.float32)
    for k in range(n):
        e = np.zeros(n, np.float32)
        e[k] = 1.0
        m1[:, k] = O.dct1d(e)
    inp = _lcg_block(n * n).reshape(n, n)
    col = (m1.astype(np.float64) @ inp.astype(np.float64))          # col[j][u]
    ref = (m1.astype(np.float64) @ col.T.astype(np.float64)) / (n * n)  # ref[u][v]
    out, _ = O.dct(name, inp)
    assert np.abs(out.reshape(n, n) - ref).max() < 1e-5


@pytest.mark.parametrize("name", ["8x16", "16x8", "16x16", "16x32", "32x16", "32x32",
                                  "32x8", "8x32", "64x64", "64x32", "32x64"])
def test_dc_of_a_constant_block_is_the_8x8_dc(name):
    # src/dct.rs:3185-3213 (32x16 / 16x32; the other sizes alike): every
    # covered block's DC equals the 8x8 DCT's DC of the same constant
    _, w, h, _ = O.DCT_KINDS[name]
    _, d8 = O.dct("8x8", np.full((8, 8), 2.3, np.float32))
    _, dc = O.dct(name, np.full((h, w), 2.3, np.float32))
    assert np.abs(dc - d8[0]).max() < 1e-3


def test_rectangular_dc_follows_the_halves():
    # a block whose halves differ: the DC pair of 8x16 (left/right) and 16x8
    # (top/bottom) orders the halves' means
    a = np.zeros((8, 16), np.float32)
    a[:, 8:] = 1.0
    _, dc = O.dct("8x16", a)
    assert dc[0] < dc[1]
    _, dc = O.dct("16x8", a.T.copy())
    assert dc[0] < dc[1]


@pytest.mark.parametrize("name", ["8x8", "8x16", "16x8", "16x16", "16x32", "32x16", "32x32",
                                  "32x8", "8x32"])
def test_transforms_round_trip(name):
    # src/dct.rs:2916-2926 (and the other round-trip tests): the inverse of
    # each transform gives back the samples ((i * 53) % 97 / 97) within 1e-4
    _, w, h, _ = O.DCT_KINDS[name]
    px = (np.array([(i * 53) % 97 for i in range(w * h)], np.float32) / np.float32(97.0)).reshape(h, w)
    coeffs, _ = O.dct(name, px)
    back = O.idct(name, coeffs)
    assert np.abs(back - px).max() < 1e-4


def _pattern(fn):
    return np.array([fn(float(i % 8), float(i // 8)) for i in range(64)], np.float32)


@pytest.mark.parametrize("fwd,inv,fn", [
    # src/dct.rs:3469-3485 and :3488-3504
    ("identity", "inv_identity",
     lambda x, y: np.float32(0.31) * np.float32(x) - np.float32(0.17) * np.float32(y)
     + np.float32(math.sin(np.float32(x * y * np.float32(0.23))))),
    ("dct2x2", "inv_dct2x2",
     lambda x, y: np.float32(math.sin(np.float32(0.37) * np.float32(x) + np.float32(0.61) * np.float32(y)))
     + np.float32(0.07) * np.float32(x) * np.float32(y)),
])
def test_identity_and_dct2x2_round_trip_and_keep_the_dc(fwd, inv, fn):
    inp = _pattern(fn)
    coeffs = O.small_transform(fwd, inp)
    assert abs(float(coeffs[0]) - float(inp.sum(dtype=np.float32)) * (1.0 / 64.0)) < 1e-6
    back = O.small_transform(inv, coeffs)
    assert np.abs(back - inp).max() < 2e-6


@pytest.mark.parametrize("name", ["dct4x4", "dct4x8", "dct8x4"])
def test_dct4_family_dc_is_the_block_mean(name):
    # the quadrant / half DCs go through a Hadamard scaled to the mean, so a
    # block's first coefficient is its mean (constant and ramp blocks)
    for blk in (np.full(64, 1.75, np.float32), np.arange(64, dtype=np.float32) / np.float32(7.0)):
        c = O.small_transform(name, blk)
        assert abs(float(c[0]) - float(blk.mean())) < 1e-5, (name, c[0])


def _f32_nearest(text):
    # a decimal literal rounded once to the nearest float (ties to even)
    from fractions import Fraction
    exact = Fraction(text)
    a = np.float32(float(exact))
    cands = [np.nextafter(a, np.float32(-np.inf)), a, np.nextafter(a, np.float32(np.inf))]
    return min(cands, key=lambda c: (abs(Fraction(float(c)) - exact), f32_bits(c) & 1))


def test_afv_basis_is_the_reference_table():
    # src/afv.rs:48-180 stores [pixel][vector]; the oracle stores the transpose
    gold = np.array([_f32_nearest(t) for t in GOLD["afv_basis_transpose"]], np.float32).reshape(16, 16)
    basis = O.afv_basis()
    assert [f32_bits(v) for v in basis.T.reshape(-1)] == [f32_bits(v) for v in gold.reshape(-1)]


def test_afv_basis_is_orthonormal():
    # src/afv.rs:412-426
    b = O.afv_basis()
    for a in range(16):
        for c in range(16):
            dot = np.float32(0.0)
            for j in range(16):
                dot = np.float32(dot + b[a, j] * b[c, j])
            assert abs(float(dot) - (1.0 if a == c else 0.0)) < 1e-5, (a, c, dot)


def _afv_rnd(seed, count):
    # the AFV tests' generator (src/afv.rs:430-434)
    s, out = seed, []
    for _ in range(count):
        s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
        out.append(np.float32(s >> 8) / np.float32(1 << 24) - np.float32(0.5))
    return out


def test_afv_dc_equals_block_mean():
    # src/afv.rs:428-448: one generator across the four kinds
    vals = _afv_rnd(123456789, 256)
    for kind in range(4):
        inp = np.array(vals[kind * 64:(kind + 1) * 64], np.float32)
        mean = np.float32(0.0)
        for v in inp:
            mean = np.float32(mean + v)
        mean = np.float32(mean / np.float32(64.0))
        out = O.small_transform(f"afv{kind}", inp)
        assert abs(float(out[0]) - float(mean)) < 1e-5, (kind, out[0], mean)


def _numeric_inverse(n, forward):
    m = np.zeros((n, n), np.float64)
    for i in range(n):
        e = np.zeros(n, np.float32)
        e[i] = 1.0
        m[:, i] = forward(e).astype(np.float64)
    return np.linalg.inv(m)


def _afv_to_pixels(kind, c):
    # the decoder's AFV inverse as the reference's test restates it
    # (src/afv.rs:505-589): inverse AFV of the (even, even) positions, inverse
    # DCT4x4 of (even, odd), inverse DCT4x8 of the odd rows, from the
    # un-mixed sub-part DCs; the DCT4 inverses are numeric
    afv_x, afv_y = kind & 1, kind >> 1
    b00, b01, b10 = c[0], c[1], c[8]
    dcs = [np.float32((b00 + b10 + b01) * np.float32(4.0)), np.float32(b00 + b10 - b01),
           np.float32(b00 - b10)]
    px = np.full(64, np.nan, np.float32)
    coeff = np.array([c[iy * 16 + ix * 2] for iy in range(4) for ix in range(4)], np.float32)
    coeff[0] = dcs[0]
    quad = (O.afv_basis().T.astype(np.float64) @ coeff.astype(np.float64)).astype(np.float32)
    for iy in range(4):
        for ix in range(4):
            sy = 3 - iy if afv_y else iy
            sx = 3 - ix if afv_x else ix
            px[(iy + afv_y * 4) * 8 + afv_x * 4 + ix] = quad[sy * 4 + sx]
    blk = np.array([c[iy * 16 + ix * 2 + 1] for iy in range(4) for ix in range(4)], np.float32)
    blk[0] = dcs[1]
    qp = (_numeric_inverse(16, O.dct4_2d) @ blk.astype(np.float64)).astype(np.float32)
    qx = 0 if afv_x else 4
    for iy in range(4):
        px[(afv_y * 4 + iy) * 8 + qx:(afv_y * 4 + iy) * 8 + qx + 4] = qp[iy * 4:iy * 4 + 4]
    half = np.array([c[(1 + iy * 2) * 8 + ix] for iy in range(4) for ix in range(8)], np.float32)
    half[0] = dcs[2]
    hp = (_numeric_inverse(32, O.dct4_2d) @ half.astype(np.float64)).astype(np.float32)
    hy = 0 if afv_y else 4
    px[hy * 8:hy * 8 + 32] = hp
    return px


def test_afv_round_trips_through_the_decoder_reference():
    # src/afv.rs:591-614
    vals = _afv_rnd(987654321, 256)
    for kind in range(4):
        inp = np.array(vals[kind * 64:(kind + 1) * 64], np.float32)
        coeffs = O.small_transform(f"afv{kind}", inp)
        back = _afv_to_pixels(kind, coeffs)
        assert np.abs(back - inp).max() < 1e-4, (kind, np.abs(back - inp).max())


def test_dct64_round_trips():
    # src/dct.rs:2999-3014 (64x64, 1e-4) and :3072-3097 (64x32 and 32x64, 2e-4)
    y, x = np.mgrid[0:64, 0:64]
    xf, yf = x.astype(np.float32), y.astype(np.float32)
    sq = (np.float32(0.01) * xf + np.float32(0.003) * yf
          + ((x // 8 + y // 8) % 3).astype(np.float32) * np.float32(0.05)).astype(np.float32)
    c, _ = O.dct("64x64", sq)
    assert np.abs(O.idct("64x64", c) - sq).max() < 1e-4
    tall = (np.float32(0.01) * xf[:, :32] + np.float32(0.003) * yf[:, :32]).astype(np.float32)
    c, _ = O.dct("64x32", tall)
    assert np.abs(O.idct("64x32", c) - tall).max() < 2e-4
    wide = (np.float32(0.004) * xf[:32] + np.float32(0.007) * yf[:32]).astype(np.float32)
    c, _ = O.dct("32x64", wide)
    assert np.abs(O.idct("32x64", c) - wide).max() < 2e-4


def test_rectangular_dct64_constant_dc_extracts():
    # src/dct.rs:3100-3113
    for name in ("64x32", "32x64"):
        _, w, h, _ = O.DCT_KINDS[name]
        _, dc = O.dct(name, np.full((h, w), 1.5, np.float32))
        assert dc.size == 32 and np.abs(dc - 1.5).max() < 2e-4


def test_dct32x8_dc_matches_the_wider_transforms():
    # src/dct.rs:2880-2912: a 32x8 block's four DC values equal those of the
    # 32x16 block made by repeating it sideways, and of its transpose as 8x32
    half = np.array([(((i // 8) * 37) % 101) / 101.0 - 0.3 for i in range(256)], np.float32)
    _, dc = O.dct("32x8", half.reshape(32, 8))
    wide = np.array([half[(i // 16) * 8 + (i % 16) % 8] for i in range(512)], np.float32)
    _, dc16 = O.dct("32x16", wide.reshape(32, 16))
    for row in range(4):
        assert abs(dc[row] - dc16[row * 2]) < 1e-4 and abs(dc[row] - dc16[row * 2 + 1]) < 1e-4
    transposed = np.array([half[(i % 32) * 8 + i // 32] for i in range(256)], np.float32)
    _, dc_wide = O.dct("8x32", transposed.reshape(8, 32))
    assert np.abs(dc - dc_wide).max() < 1e-4


@pytest.mark.parametrize("name", ["8x16", "16x8", "16x16", "16x32", "32x16", "32x32",
                                  "32x8", "8x32", "64x64", "64x32", "32x64",
                                  "128x128", "128x64", "64x128"])
def test_dc_grid_follows_the_block_means(name):
    # on a ramp the DC values approximate the covered 8x8 blocks' means in
    # raster order of the blocks (a transposed grid would be off by 0.2+)
    _, w, h, _ = O.DCT_KINDS[name]
    y, x = np.mgrid[0:h, 0:w]
    blk = (np.float32(0.01) * x + np.float32(0.03) * y).astype(np.float32)
    _, dc = O.dct(name, blk)
    means = blk.reshape(h // 8, 8, w // 8, 8).mean(axis=(1, 3)).reshape(-1)
    assert np.abs(dc - means).max() < 0.01


def _pattern128(w, h):
    # src/dct128.rs:945-957
    y, x = np.mgrid[0:h, 0:w]
    return (np.float32(0.01) * x.astype(np.float32) + np.float32(0.003) * y.astype(np.float32)
            + ((x // 8 + 2 * (y // 8)) % 5).astype(np.float32) * np.float32(0.05)
            + ((x * 7 + y * 13) % 11).astype(np.float32) * np.float32(0.002)).astype(np.float32)


@pytest.mark.parametrize("name", ["128x128", "128x64", "64x128"])
def test_dct128_round_trips(name):
    # src/dct128.rs:976-1010
    _, w, h, _ = O.DCT_KINDS[name]
    px = _pattern128(w, h)
    c, _ = O.dct(name, px)
    assert np.abs(O.idct(name, c) - px).max() < 2e-4


@pytest.mark.parametrize("name", ["128x128", "128x64", "64x128"])
def test_dct128_dc_grid_tracks_block_means_on_smooth_content(name):
    # src/dct128.rs:1012-1063: tall and wide blocks are the top-left part of
    # the 128x128 image
    y, x = np.mgrid[0:128, 0:128]
    img = np.array([math.sin(np.float32(v)) for v in (x * np.float32(0.021)).reshape(-1)],
                   np.float32).reshape(128, 128)
    img = (img + np.array([math.cos(np.float32(v)) for v in (y * np.float32(0.013)).reshape(-1)],
                          np.float32).reshape(128, 128) * np.float32(0.5)).astype(np.float32)
    _, w, h, _ = O.DCT_KINDS[name]
    blk = np.ascontiguousarray(img[:h, :w])
    _, dc = O.dct(name, blk)
    means = blk.reshape(h // 8, 8, w // 8, 8).mean(axis=(1, 3)).reshape(-1)
    assert np.abs(dc - means).max() < 0.02


@pytest.mark.parametrize("name", ["128x128", "128x64", "64x128", "64x64", "64x32", "32x64"])
def test_large_dct_cosine_basis(name):
    # src/dct128.rs:851-886: a separable cosine of frequencies (u, v) lands on
    # one coefficient, 1 / sqrt(2) per non-zero frequency, at u H + v when
    # H >= W, else v W + u
    _, w, h, _ = O.DCT_KINDS[name]
    for u, v in [(0, 0), (1, 0), (0, 1), (w // 2, h // 2), (w - 3, h - 3), (w - 1, h - 1)]:
        i = np.arange(w * h)
        xs = np.cos((math.pi * (i % w) + math.pi / 2) * u / w)
        ys = np.cos((math.pi * (i // w) + math.pi / 2) * v / h)
        px = (xs * ys).astype(np.float32).reshape(h, w)
        got, _ = O.dct(name, px)
        want = np.zeros(w * h, np.float32)
        index = u * h + v if h >= w else v * w + u
        want[index] = (1.0 if u == 0 else np.float32(math.sqrt(0.5))) * (
            1.0 if v == 0 else np.float32(math.sqrt(0.5)))
        assert np.abs(got - want).max() < 2e-6, (name, u, v, np.abs(got - want).max())


def test_transfer_tables_follow_transfer_lut_build():
    # TransferLut::build (src/color.rs:297-333): 8-bit sRGB is the f64
    # table; other depths decode v / max in f32 over a 65536-entry domain,
    # codes above the largest decoding to 0
    s8 = O.transfer_lut(8, 13)
    assert np.array_equal(s8, O.transfer_lut(8, 0))
    ref = np.zeros(256, np.float32)
    O.lib().orc_srgb_lut(ref.ctypes.data_as(__import__("ctypes").c_void_p))
    assert np.array_equal(s8, ref)
    for bits in (10, 12, 16):
        mx = (1 << bits) - 1
        v = np.arange(mx + 1, dtype=np.float64) / mx
        f64 = {  # the formulas of src/color.rs:44-199 in float64
            13: np.where(v <= 0.04045, v / 12.92, ((v + 0.055) / 1.055) ** 2.4),
            8: v,
            1: np.where(v < 4.5 * 0.01805397, v / 4.5, ((v + 0.0992968) / 1.0992968) ** (1 / 0.45)),
            4: v ** 2.2, 5: v ** 2.8, 17: v ** 2.6,
            7: np.where(v < 0.0912, v / 4.0, ((v + 0.1115) / 1.1115) ** (1 / 0.45)),
        }
        for tf, want in f64.items():
            t = O.transfer_lut(bits, tf)
            assert t.size == 65536 and t[0] == 0.0 and abs(float(t[mx]) - 1.0) < 1e-6, (bits, tf)
            assert np.abs(t[: mx + 1] - want).max() < 2e-6, (bits, tf)
            assert not np.any(t[mx + 1:]), (bits, tf)
        # linear is the f32 quotient itself
        lin = (np.arange(mx + 1, dtype=np.float32) / np.float32(mx)).astype(np.float32)
        assert np.array_equal(O.transfer_lut(bits, 8)[: mx + 1], lin)
    # the 8-bit non-default transfers take the f32 formula too
    v = np.arange(256, dtype=np.float64) / 255
    bt709 = np.where(v < 4.5 * 0.01805397, v / 4.5, ((v + 0.0992968) / 1.0992968) ** (1 / 0.45))
    assert np.abs(O.transfer_lut(8, 1) - bt709).max() < 1e-6


def test_transfer_codes_the_front_end_rejects():
    for tf in (16, 18, 3, 19, -1):
        with pytest.raises(ValueError):
            O.transfer_lut(16, tf)
    with pytest.raises(ValueError):
        O.transfer_lut(9, 13)


def test_high_depth_samples_above_the_largest_code():
    # 10-bit: a sample above 1023 decodes to 0 (its LUT slot is empty), and
    # an alpha above 1023 is capped to it
    rng = np.random.default_rng(5)
    img = rng.integers(0, 1024, (24, 24, 4)).astype(np.uint16)
    img[..., 3] = 1023
    hi = img.copy()
    hi[3, 4, 0] = 4000
    zero = img.copy()
    zero[3, 4, 0] = 0
    hi[..., 3][hi[..., 3] == 1023] = 60000
    a = O.frontend(hi, 1.0, bits=10)
    b = O.frontend(zero, 1.0, bits=10)
    assert np.array_equal(a.xyb, b.xyb)
    assert np.array_equal(a.alpha, np.full((24, 24), 1023, np.uint16))
    assert a.tokens.tolist() == b.tokens.tolist()


def test_grey_is_snapped_achromatic():
    # linearize_gray (src/encode_image.rs:1571-1600) writes the decoded luma
    # to all three planes, and the grey encode is achromatic
    # (with_grayscale(true), src/encode_image.rs:3968), so encode_frame snaps
    # the XYB planes after the conversion and the invisible fill:
    # X = 0 and B = Y exactly (snap_achromatic_xyb, src/frame/encoder.rs:155-157,
    # :351-357).  The RGB frame (g, g, g) is not snapped: its X plane holds the
    # rounding noise of the three opsin mixes.
    from jixel_gb300 import synthetic
    img = synthetic.generate(72, 40, 9, alpha=True)
    g, a = img[..., 1], img[..., 3]
    grey, rgb = O.frontend(g, 1.0), O.frontend(np.stack([g, g, g], -1), 1.0)
    assert np.all(grey.xyb[0] == 0.0) and not np.signbit(grey.xyb[0]).any()
    assert np.array_equal(grey.xyb[2], grey.xyb[1])
    assert np.array_equal(grey.xyb[1], rgb.xyb[1])
    assert not np.array_equal(grey.xyb, rgb.xyb)
    # grey + alpha takes its alpha from the second channel; the snap follows
    # the fill
    ga, rgba = O.frontend(np.stack([g, a], -1), 1.0), O.frontend(np.stack([g, g, g, a], -1), 1.0)
    assert np.array_equal(ga.alpha, rgba.alpha)
    assert np.all(ga.xyb[0] == 0.0) and np.array_equal(ga.xyb[2], ga.xyb[1])
    assert np.array_equal(ga.xyb[1], rgba.xyb[1])
