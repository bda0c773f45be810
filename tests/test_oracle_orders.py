"""Coefficient-order statistics: the restatement (oracle/coeff_order.py)
pinned to the reference's own tests of src/coeff_order.rs (:715-840) and to
its tables, then the library's host-side derive_orders (jxg_derive_orders,
no device) checked against it on synthetic statistics."""
import json
import os

import numpy as np
import pytest

import jixel_gb300 as J
from oracle import coeff_order as C
from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tables.json")))


def test_tables_are_the_reference_tables():
    assert C.STRATEGY_CODE_LUT == GOLD["strategy_code_lut"]
    assert C.K_STRATEGY_ORDER == GOLD["strategy_order"]
    # the strategies a frame holds: DCT8, 16x8 / 8x16, 16x16, 32x32
    assert [C.slot_of(s) for s in range(5)] == [0, 4, 4, 2, 3]
    assert list(J.api.ORDER_SLOT_SIZES) == [size for (_, _, size) in C.ORDER_SPECS]


def test_generic_natural_scan_reproduces_the_spec_tables():
    # generic_natural_scan_reproduces_the_spec_tables (src/coeff_order.rs:719-743)
    assert O.natural_scan(4, 2).tolist() == GOLD["coeff_order_32x16"]
    assert O.natural_scan(2, 1).tolist() == GOLD["coeff_order_16x8"]
    assert O.natural_scan(2, 2).tolist() == GOLD["coeff_order_16x16"]
    scan = O.natural_scan(4, 1)
    assert scan[:4].tolist() == [0, 1, 2, 3]
    assert sorted(scan.tolist()) == list(range(256))


def _lcg_shuffle(n, state):
    perm = list(range(n))
    for i in range(n - 1, 0, -1):
        state = (state * 1664525 + 1013904223) & 0xFFFFFFFF
        j = (state >> 8) % (i + 1)
        perm[i], perm[j] = perm[j], perm[i]
    return perm, state


def test_lehmer_code_round_trips():
    # lehmer_code_round_trips (src/coeff_order.rs:745-763)
    state = 12345
    for n in (4, 16, 64, 128):
        perm, state = _lcg_shuffle(n, state)
        assert C.lehmer_decode(C.lehmer_code(perm)) == perm, n


def test_natural_order_tokenizes_to_one_token():
    # natural_order_tokenizes_to_one_token (src/coeff_order.rs:765-773)
    tokens = C.permutation_tokens(list(range(64)), 1)
    assert len(tokens) == 1 and tokens[0][1] == 0


def test_coeff_order_context_matches_libjxl():
    # coeff_order_context_matches_libjxl (src/coeff_order.rs:776-787)
    for v, want in [(0, 0), (1, 1), (2, 2), (3, 2), (4, 3), (7, 3), (8, 4), (1 << 6, 7), (1 << 20, 7)]:
        assert C.coeff_order_context(v) == want, v


def test_derive_is_the_stable_frequency_order():
    # packed_coefficient_order_matches_stable_frequency_order (src/coeff_order.rs:789-838)
    rng = 0x93AB2017
    for n in (1, 2, 7, 64, 128, 4096):
        natural = list(range(n))
        for i in range(n - 1, 0, -1):
            rng = (rng * 1664525 + 1013904223) & 0xFFFFFFFF
            j = rng % (i + 1)
            natural[i], natural[j] = natural[j], natural[i]
        for pattern in range(4):
            counts = []
            for i in range(n):
                if pattern == 0:
                    counts.append(0)
                elif pattern == 1:
                    counts.append(0xFFFFFFFF)
                elif pattern == 2:
                    counts.append(i % 7)
                else:
                    rng = (rng * 1664525 + 1013904223) & 0xFFFFFFFF
                    counts.append(rng)
            counts = np.array(counts, np.uint64)
            for llf in (0, 1, n // 3, n):
                expected = natural[:llf] + sorted(natural[llf:], key=lambda r: -int(counts[r]))
                assert C.derive(counts, natural, llf) == expected, (n, llf, pattern)


def _stats(seed, blocks, skew):
    """Synthetic statistics: per slot and channel, non-zero counts that fall
    off along a shuffled frequency ranking (`skew` how much the natural scan
    differs from it)."""
    rng = np.random.default_rng(seed)
    counts = []
    for slot, (_, _, size) in enumerate(C.ORDER_SPECS):
        per = np.zeros((3, size), np.uint32)
        for c in range(3):
            rank = np.arange(size, dtype=np.float64)
            rank = rank + skew * rng.normal(0, size / 8, size)
            p = np.exp(-rank / (size / 10))
            per[c] = np.minimum(rng.binomial(blocks[slot], np.clip(p, 0, 1)), blocks[slot]).astype(np.uint32)
        counts.append(per)
    return counts


@pytest.mark.parametrize("seed,skew", [(1, 0.0), (2, 0.5), (3, 2.0), (4, 6.0)])
def test_library_derive_orders_matches_the_restatement(seed, skew):
    blocks = [5000, 30, 900, 200, 63, 64, 70]
    counts = _stats(seed, blocks, skew)
    used, orders, moved = J.derive_orders(counts, blocks)
    want_used, want_orders, want_moved = C.derive_orders(counts, blocks)
    assert used == want_used
    assert moved == want_moved
    for slot in range(len(C.ORDER_SPECS)):
        assert np.array_equal(orders[slot], np.array(want_orders[slot], np.uint32)), slot


def test_derive_orders_gates():
    # a slot below MIN_BLOCKS_FOR_ORDER keeps its natural order; statistics
    # that already follow the natural order adopt nothing and move nothing
    counts = _stats(7, [63] * 7, 4.0)
    used, orders, moved = J.derive_orders(counts, [63] * 7)
    assert used == 0 and moved == 0.0
    for slot in range(len(C.ORDER_SPECS)):
        assert all(np.array_equal(orders[slot][c], C.natural_order(slot)) for c in range(3))
    natural_counts = []
    for slot, (_, llf, size) in enumerate(C.ORDER_SPECS):
        nat = C.natural_order(slot)
        per = np.zeros((3, size), np.uint32)
        per[:, nat] = np.arange(size, 0, -1, dtype=np.uint32)  # falls off along the natural scan
        natural_counts.append(per)
    used, _, moved = J.derive_orders(natural_counts, [10000] * 7)
    assert used == 0 and moved == 0.0
    # strongly skewed statistics adopt an order
    used, _, moved = J.derive_orders(_stats(8, [20000] * 7, 6.0), [20000] * 7)
    assert used != 0 and 0.0 < moved < 1.0


def test_derive_orders_rejects_bad_arguments():
    with pytest.raises(J.EncodeError):
        J.derive_orders([np.zeros((3, 64), np.uint32)], [0])
