"""Bit-exact comparison of one front-end result with the oracle's."""
import numpy as np


def assert_same(got, want, check_xyb=True):
    p = got.params
    for k in ("global_scale", "quant_dc", "x_qm_scale", "b_qm_scale", "epf_iters"):
        assert p[k] == want.params[k], k
    assert p["scale"] == want.params["scale"] and p["scale_dc"] == want.params["scale_dc"]
    assert p["dc_step"] == want.params["dc_step"]
    if check_xyb:
        assert np.array_equal(got.xyb.view(np.uint32), want.xyb.view(np.uint32)), "xyb"
    assert p["constant_blocks"] == want.constant_blocks
    assert p["screen_content"] == want.screen_content
    assert p["epf_sharpness"] == want.epf_sharpness
    assert np.array_equal(got.quant_field, want.quant_field), "quant field"
    assert p["qf_threshold"] == want.qf_threshold
    assert np.array_equal(got.ytox, want.ytox), "ytox"
    assert np.array_equal(got.ytob, want.ytob), "ytob"
    assert np.array_equal(got.quant_dc, want.quant_dc), "quant_dc"
    if got.coefficients is not None:
        assert np.array_equal(got.coefficients, want.coeffs), "coefficients"
    assert np.array_equal(got.num_nzeros, want.nzeros), "nzeros"
    assert np.array_equal(got.group_offsets, want.group_offsets), "group offsets"
    assert got.tokens.shape == want.tokens.shape, "token count"
    assert np.array_equal(got.tokens, want.tokens), "tokens"
    assert np.array_equal(got.histograms, want.histograms), "histograms"
    assert np.array_equal(got.ac_strategy, want.ac_strategy), "ac_strategy"
    if getattr(want, "alpha", None) is not None and getattr(got, "alpha", None) is not None:
        assert np.array_equal(got.alpha, want.alpha), "alpha"


def high_depth_image(w, h, seed, bits, alpha=False):
    """Synthetic content scaled to `bits` in uint16 words, plus a few samples
    above the largest code (they decode to 0; alpha above it is capped)."""
    from jixel_gb300 import synthetic
    img = synthetic.generate(w, h, seed, sixteen_bit=True, alpha=alpha).astype(np.uint32)
    img = (img * ((1 << bits) - 1) // 65535).astype(np.uint16)
    if bits < 16:
        rng = np.random.default_rng(seed)
        ys, xs = rng.integers(0, h, 40), rng.integers(0, w, 40)
        img[ys, xs, rng.integers(0, img.shape[2], 40)] = (1 << bits) + 7
    return img
