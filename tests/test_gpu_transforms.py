"""The operator table's larger transforms (DctFn<W, H, N> of src/dct.rs) and
their DC extraction, bit-exact against the oracle's restatement."""
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


ALL_DCT = ["8x8", "8x16", "16x8", "16x16", "16x32", "32x16", "32x32", "32x8", "8x32",
           "64x64", "64x32", "32x64", "128x128", "128x64", "64x128"]


@pytest.mark.parametrize("name", ALL_DCT)
def test_transform_and_dc_match_oracle(ctx, name):
    _, w, h, ndc = O.DCT_KINDS[name]
    rng = np.random.default_rng(w * 100 + h)
    blocks = rng.uniform(-1.0, 1.0, (150, h, w)).astype(np.float32)
    blocks[0] = 0.37                                   # constant
    blocks[1] = np.linspace(0.0, 1.0, w, dtype=np.float32)[None, :]  # horizontal ramp
    blocks[2] = np.linspace(0.0, 1.0, h, dtype=np.float32)[:, None]  # vertical ramp
    blocks[3] *= 1e-6                                  # tiny values
    blocks[4] *= 1e4                                   # large values
    got, dc = ctx.dct(name, blocks)
    for i, b in enumerate(blocks):
        want, want_dc = O.dct(name, b)
        assert np.array_equal(got[i].view(np.uint32), want.view(np.uint32)), (name, i)
        assert np.array_equal(dc[i].view(np.uint32), want_dc.view(np.uint32)), (name, i)


def test_dct_operator_rejects_bad_kinds(ctx):
    lib = ctx._lib
    b = np.zeros(64, np.float32)
    assert lib.jxg_op_dct(ctx.handle, 15, b.ctypes.data, 1, b.ctypes.data, None) != 0
    assert lib.jxg_op_idct(ctx.handle, 15, b.ctypes.data, 1, b.ctypes.data) != 0
    assert lib.jxg_op_small_transform(ctx.handle, 11, b.ctypes.data, 1, b.ctypes.data) != 0
    assert lib.jxg_op_dct(ctx.handle, -1, b.ctypes.data, 1, b.ctypes.data, None) != 0
    assert lib.jxg_op_dct(ctx.handle, 3, b.ctypes.data, 0, b.ctypes.data, None) == 0  # no blocks


@pytest.mark.parametrize("name", ALL_DCT)
def test_inverse_matches_oracle_and_round_trips(ctx, name):
    _, w, h, _ = O.DCT_KINDS[name]
    rng = np.random.default_rng(w * 7 + h)
    blocks = rng.uniform(-1.0, 1.0, (120, h, w)).astype(np.float32)
    coeffs, _ = ctx.dct(name, blocks)
    back = ctx.idct(name, coeffs)
    for i in range(blocks.shape[0]):
        want = O.idct(name, coeffs[i])
        assert np.array_equal(back[i].view(np.uint32), want.view(np.uint32)), (name, i)
    assert np.abs(back - blocks).max() < 1e-4


@pytest.mark.parametrize("name", ["identity", "dct2x2", "dct4x4", "dct4x8", "dct8x4",
                                  "inv_identity", "inv_dct2x2", "afv0", "afv1", "afv2", "afv3"])
def test_small_transforms_match_oracle(ctx, name):
    rng = np.random.default_rng(len(name) * 31)
    blocks = rng.uniform(-1.0, 1.0, (300, 8, 8)).astype(np.float32)
    blocks[0] = 0.5
    blocks[1] *= 1e5
    got = ctx.small_transform(name, blocks)
    for i, b in enumerate(blocks):
        want = O.small_transform(name, b)
        assert np.array_equal(got[i].view(np.uint32), want.view(np.uint32)), (name, i)
