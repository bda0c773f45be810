"""The allocation-free token-offset entry point against the front end's own.

`jxg_token_offsets_noalloc` serves callers that cannot allocate device
memory while encoding (their own pool owns every buffer, or allocation is
forbidden after start-up); it must place tokens exactly where the ordinary
front end (`jxg_frontend`, which allocates its scratch per context) places
them.  Token offsets are integers, so the check is exact.  Two calls in a
row on different frames also show that the shared scratch array carries
nothing from one call into the next.  This file sorts last so a run that
stops at the first failure has already run every other test.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import _lib as L
from jixel_gb300 import synthetic

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tables.json")))


def token_counts(res, width, height):
    """Tokens per (block, channel) in the [group][1024][Y, X, B] layout."""
    scan = np.array(GOLD["coeff_order_8x8"])
    position = np.zeros(64, np.int64)
    position[scan] = np.arange(64)
    fi = J.frame_info(width, height)
    counts = np.zeros((fi.num_groups, 1024, 3), np.uint32)
    coeffs = res.coefficients  # (yb, xb, 3 [X, Y, B], 64)
    nonzero = coeffs != 0
    nonzero[..., 0] = False
    last = np.where(nonzero, position[None, None, None, :], 0).max(-1)  # (yb, xb, 3)
    per = 1 + last
    order = [1, 0, 2]  # tokens go Y, X, B
    for by in range(fi.ysize_blocks):
        for bx in range(fi.xsize_blocks):
            g = (by // 32) * fi.xsize_groups + bx // 32
            lb = (by % 32) * 32 + bx % 32
            counts[g, lb, :] = per[by, bx, order]
    return counts


def run_noalloc(counts, num_groups, stream):
    import torch

    d_counts = torch.from_numpy(counts.reshape(-1).view(np.int32)).cuda()
    d_offsets = torch.zeros_like(d_counts)
    d_groups = torch.zeros(num_groups + 1, dtype=torch.int64, device="cuda")
    lib = L.load()
    st = lib.jxg_token_offsets_noalloc(d_counts.data_ptr(), num_groups, d_offsets.data_ptr(),
                                       d_groups.data_ptr(), stream.cuda_stream)
    assert st == 0, st
    stream.synchronize()
    return (d_offsets.cpu().numpy().view(np.uint32).reshape(counts.shape),
            d_groups.cpu().numpy().view(np.uint64))


def test_noalloc_offsets_match_frontend_twice():
    torch = pytest.importorskip("torch")
    ctx = J.FrontendContext(0)
    stream = torch.cuda.Stream()
    cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90)
    try:
        for (w, h, seed) in [(700, 520, 91), (300, 260, 92)]:
            img = synthetic.generate(w, h, seed, rectangles=6)
            res = ctx.frontend(img, cfg)
            fi = J.frame_info(w, h)
            counts = token_counts(res, w, h)
            offsets, groups = run_noalloc(counts, fi.num_groups, stream)
            # per-group offsets and the total equal the front end's
            assert np.array_equal(groups, res.group_offsets)
            assert int(groups[-1]) == res.tokens.shape[0]
            # every entry offset lands on that block-channel's non-zero-count token
            nz = res.num_nzeros  # (3, yb, xb), X Y B
            for by in range(fi.ysize_blocks):
                for bx in range(fi.xsize_blocks):
                    g = (by // 32) * fi.xsize_groups + bx // 32
                    lb = (by % 32) * 32 + bx % 32
                    for co, c in enumerate((1, 0, 2)):
                        tok = res.tokens[offsets[g, lb, co]]
                        assert tok[1] == nz[c, by, bx]
    finally:
        ctx.close()


def test_noalloc_rejects_oversized_requests():
    lib = L.load()
    assert lib.jxg_token_offsets_noalloc(None, 1, None, None, None) == 100
    # beyond the stated limit: a clear size error before touching any pointer
    big = L.NOALLOC_MAX_GROUPS + 1
    assert lib.jxg_token_offsets_noalloc(ctypes.c_void_p(16), big, ctypes.c_void_p(16),
                                         ctypes.c_void_p(16), None) == 6
