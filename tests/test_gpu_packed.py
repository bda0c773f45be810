"""The groups' token storage form (AcTokens, src/entropy/token_stream.rs:37-76).

PendingAcGroup holds each group's tokens as one 32-bit word per token
(context << 18 | value) unless a context or value of the group is out of
that range, in which case the group keeps (context, value) pairs.  The
device writes that form straight from the token stream; it must equal the
oracle's per-group restatement of AcTokens::from on the oracle's tokens,
through the synchronous, asynchronous and batch paths and through the
operator entry point (whose inputs reach the wide form).
"""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic
from jixel_gb300.api import unpack_tokens
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def ultrafast(d):
    return J.EncodeConfig(distance=d, speed=J.Speed.ULTRA_FAST)


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def check_packed(r, tokens, goffs):
    words, woffs = O.ac_tokens_from(tokens, goffs)
    assert np.array_equal(r.packed_offsets, woffs)
    assert np.array_equal(r.packed_tokens, words)
    assert np.array_equal(unpack_tokens(r.packed_tokens, r.packed_offsets, r.group_offsets),
                          tokens)


@pytest.mark.parametrize("shape,kw,d", [
    ((320, 200), {}, 1.0),
    ((700, 530), {"rectangles": 40}, 0.2783),   # 3x3 groups, ragged
    ((257, 300), {"alpha": True}, 2.35),
    ((513, 129), {"sixteen_bit": True}, 1.45),
    ((1, 1), {}, 1.0),
])
def test_frontend_packed_tokens_match_oracle(ctx, shape, kw, d):
    img = synthetic.generate(*shape, 91, **kw)
    want = O.frontend(img, d)
    r = ctx.frontend(img, ultrafast(d), packed=True)
    assert np.array_equal(r.tokens, want.tokens)
    assert np.array_equal(r.group_offsets, want.group_offsets)
    check_packed(r, want.tokens, want.group_offsets)
    assert int(r.packed_offsets[-1]) == len(want.tokens)  # 8/16-bit input never goes wide


def test_async_packed_outputs(ctx):
    torch = pytest.importorskip("torch")
    imgs = [synthetic.generate(384, 272, 92 + i) for i in range(3)]
    out = J.PinnedOutputs(384, 272, packed=True)
    assert out.tokens is None
    pix = torch.empty((272, 384, 3), dtype=torch.uint8, pin_memory=True).numpy()
    for img in imgs:
        pix[:] = img
        ctx.enqueue(pix, ultrafast(1.0), out)
        ctx.wait()
        r = out.result()
        want = O.frontend(img, 1.0)
        assert r.params["num_tokens"] == len(want.tokens)
        assert np.array_equal(r.group_offsets, want.group_offsets)
        check_packed(r, want.tokens, want.group_offsets)


def test_async_packed_capacity_is_checked(ctx):
    pytest.importorskip("torch")
    img = synthetic.generate(200, 120, 93)
    out = J.PinnedOutputs(200, 120, packed=True)
    out.c.packed_capacity = 10  # far fewer words than the frame's tokens
    ctx.enqueue(img, ultrafast(1.0), out)
    with pytest.raises(J.EncodeError):
        ctx.wait()


def test_batch_packed_results(ctx):
    imgs = [synthetic.generate(300, 200, 94), synthetic.generate(90, 70, 95, alpha=True),
            synthetic.generate(520, 260, 96, sixteen_bit=True)]
    b = ctx.batch()
    try:
        for img in imgs:
            b.add(img, ultrafast(1.0))
        b.run(use_graph=True)
        for i, img in enumerate(imgs):
            want = O.frontend(img, 1.0)
            check_packed(b.result(i, packed=True), want.tokens, want.group_offsets)
    finally:
        b.close()


def _op_case(rng, groups, wide_groups, max_len=300):
    lens = rng.integers(0, max_len, groups)
    goffs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    n = int(goffs[-1])
    toks = np.stack([rng.integers(0, 14850, n), rng.integers(0, 1 << 18, n)], 1).astype(np.uint32)
    for g in wide_groups:
        if lens[g]:
            k = int(goffs[g]) + int(rng.integers(0, lens[g]))
            if rng.integers(0, 2):
                toks[k, 1] = np.uint32(1 << 18) + np.uint32(rng.integers(0, 1 << 20))
            else:
                toks[k, 0] = np.uint32(1 << 14) + np.uint32(rng.integers(0, 1 << 10))
    return toks, goffs


def test_pack_op_reference_boundaries(ctx):
    mc, mv = O.PACKED_MAX_CONTEXT, O.PACKED_MAX_VALUE
    source = [[0, 0], [mc, mv], [O.NUM_FINE_AC_CONTEXTS - 1, 31]]
    for extra in ([], [[0, mv + 1]], [[mc + 1, 0]], [[0xFFFFFFFF, 0xFFFFFFFF]]):
        toks = np.array(source + extra, np.uint64).astype(np.uint32)
        goffs = np.array([0, len(toks)], np.uint64)
        words, woffs = ctx.pack_tokens(toks, goffs)
        want_w, want_o = O.ac_tokens_from(toks, goffs)
        assert np.array_equal(words, want_w) and np.array_equal(woffs, want_o)


@pytest.mark.parametrize("groups,wide", [(1, []), (7, [0, 3, 6]), (135, [5, 70, 134]),
                                         (1024, list(range(0, 1024, 97)))])
def test_pack_op_mixed_groups(ctx, groups, wide):
    rng = np.random.default_rng(groups)
    toks, goffs = _op_case(rng, groups, wide)
    words, woffs = ctx.pack_tokens(toks, goffs)
    want_w, want_o = O.ac_tokens_from(toks, goffs)
    assert np.array_equal(woffs, want_o)
    assert np.array_equal(words, want_w)


def test_pack_op_more_groups_than_one_grid_row(ctx):
    # 70,000 groups: more than a grid's 65,535 rows, so CTAs loop over groups
    rng = np.random.default_rng(7)
    toks, goffs = _op_case(rng, 70000, [1, 65534, 65535, 69999], max_len=4)
    words, woffs = ctx.pack_tokens(toks, goffs)
    want_w, want_o = O.ac_tokens_from(toks, goffs)
    assert np.array_equal(woffs, want_o)
    assert np.array_equal(words, want_w)


def test_pack_op_rejects_bad_input(ctx):
    lib, h = ctx._lib, ctx.handle
    toks = np.zeros((4, 2), np.uint32)
    goffs = np.array([0, 3, 2], np.uint64)  # decreasing
    words = np.zeros(8, np.uint32)
    woffs = np.zeros(3, np.uint64)
    assert lib.jxg_op_pack_tokens(h, toks.ctypes.data, goffs.ctypes.data, 2, words.ctypes.data,
                                  8, woffs.ctypes.data) != 0
    goffs = np.array([0, 4], np.uint64)
    assert lib.jxg_op_pack_tokens(h, toks.ctypes.data, goffs.ctypes.data, 1, words.ctypes.data,
                                  2, woffs.ctypes.data) != 0  # 4 words, room for 2
    assert woffs.tolist()[:2] == [0, 4]
