"""CPU restatement of the reference's coefficient-order statistics (test
infrastructure: only the tests import it, as the checker of the library's
order-statistics kernel and of its host-side order derivation).

Pass one tallies, per order group ("slot") and channel, how many transforms
carry a non-zero level at each raw coefficient index, counted over the whole
block and not only the walked prefix (`OrderStats::tally` /
`tally_block`, src/coeff_order.rs:511-540, called by the tokeniser at
src/group.rs:2555-2574).  `derive_orders` (src/coeff_order.rs:621-673) then
proposes, per slot and channel, the scan that visits the most often
non-zero positions first (`OrderStats::derive`, :586-601) and keeps it where
the saving predicted by the expected scan walk (`expected_walk`, :570-581)
pays for the permutation's tokens (`tokenize_permutation`, :89-105, with the
Lehmer code of :54-71).  The arithmetic is the reference's: f64, sequential,
left to right.
"""
import numpy as np

from oracle import oracle as O

# ORDER_SPECS (src/coeff_order.rs:117-125): (order group, LLF entries, coefficients)
ORDER_SPECS = [(0, 1, 64), (1, 1, 64), (2, 4, 256), (3, 16, 1024), (4, 2, 128), (5, 4, 256),
               (6, 8, 512)]
# the natural order of each slot as (cx, cy) of natural_scan_generic
# (src/coeff_order.rs:210-253, CoeffOrders::natural :425-448)
SLOT_SHAPES = [(1, 1), (1, 1), (2, 2), (4, 4), (2, 1), (4, 1), (4, 2)]
# STRATEGY_CODE_LUT (src/dc_group_data.rs:79-81): raw strategy -> JXL code
STRATEGY_CODE_LUT = [0, 6, 7, 4, 5, 3, 12, 13, 10, 11, 14, 15, 16, 17, 18, 19, 20, 1, 2, 21, 22,
                     23, 8, 9]
# K_STRATEGY_ORDER (src/ac_context.rs:80-83): JXL code -> order group
K_STRATEGY_ORDER = [0, 1, 1, 1, 2, 3, 4, 4, 5, 5, 6, 6, 1, 1, 1, 1, 1, 1, 7, 8, 8, 9, 10, 10, 11,
                    12, 12]
# covered blocks (x, y) of the raw strategies a frame of this build holds
COVERED = {0: (1, 1), 1: (1, 2), 2: (2, 1), 3: (2, 2), 4: (4, 4)}

PERMUTATION_CONTEXTS = 8      # src/coeff_order.rs:34
MIN_BLOCKS_FOR_ORDER = 64     # :606
BITS_PER_SAVED_TOKEN = 0.2    # :608
GATE_MARGIN = 1.5             # :611
BITS_PER_PERMUTATION_TOKEN = 5.0  # :616


def slot_of(raw_strategy: int):
    """order_slot_of (src/coeff_order.rs:502-506) of a raw strategy."""
    group = K_STRATEGY_ORDER[STRATEGY_CODE_LUT[raw_strategy]]
    for slot, (g, _, _) in enumerate(ORDER_SPECS):
        if g == group:
            return slot
    return None


def natural_order(slot: int) -> np.ndarray:
    """Scan position -> raw index of a slot's natural order."""
    return O.natural_scan(*SLOT_SHAPES[slot]).astype(np.int64)


def natural_position(slot: int) -> np.ndarray:
    """natural_position_lut_for_order (src/coeff_order.rs:271-295): raw index
    -> natural scan position."""
    scan = natural_order(slot)
    pos = np.empty_like(scan)
    pos[scan] = np.arange(scan.size)
    return pos


def tally(coeffs: np.ndarray, strategy: np.ndarray | None):
    """OrderStats of one frame: `coeffs` (yb, xb, 3, 64) levels in raw order,
    each transform's coefficients in 64-entry chunks over its covered blocks
    (chunk k at block row k // cx, column k % cx); `strategy` (yb, xb) u8
    (raw << 1) | first, or None for an all-DCT8 frame.  Returns (counts, blocks):
    counts[slot] (3, size) u32, blocks[slot]."""
    yb, xb = coeffs.shape[:2]
    if strategy is None:
        strategy = np.ones((yb, xb), np.uint8)
    counts = [np.zeros((3, size), np.uint64) for (_, _, size) in ORDER_SPECS]
    blocks = [0] * len(ORDER_SPECS)
    first = (strategy & 1) == 1
    raw = strategy >> 1
    for st, (cx, cy) in COVERED.items():
        ys, xs = np.nonzero(first & (raw == st))
        slot = slot_of(st)
        if ys.size == 0 or slot is None:
            continue
        blocks[slot] += int(ys.size)
        chunks = [coeffs[ys + k // cx, xs + k % cx] for k in range(cx * cy)]  # each (n, 3, 64)
        levels = np.concatenate(chunks, axis=2)  # (n, 3, size): raw index k * 64 + i
        counts[slot] += np.count_nonzero(levels, axis=0).astype(np.uint64)
    return [c.astype(np.uint32) for c in counts], blocks


def coeff_order_context(val: int) -> int:
    """coeff_order_context (src/coeff_order.rs:40-48): the (0, 0, 0) hybrid-uint
    token, 0 for 0 and 1 + floor(log2(val)) otherwise, at most 7."""
    return 0 if val == 0 else min(val.bit_length(), PERMUTATION_CONTEXTS - 1)


def lehmer_code(perm) -> list[int]:
    """compute_lehmer_code (src/coeff_order.rs:54-71): code[i] = the entries
    after position i smaller than perm[i]."""
    p = np.asarray(perm, np.int64)
    return [int(np.count_nonzero(p[i + 1:] < p[i])) for i in range(p.size)]


def lehmer_decode(code) -> list[int]:
    """decode_lehmer_code (src/coeff_order.rs:79-85)."""
    available = list(range(len(code)))
    return [available.pop(c) for c in code]


def permutation_tokens(zigzag, skip: int) -> list[tuple[int, int]]:
    """tokenize_permutation (src/coeff_order.rs:89-105): (context, value)
    tokens of a permutation in natural-scan space, its first `skip` entries
    left alone."""
    lehmer = lehmer_code(zigzag)
    end = len(lehmer)
    while end > skip and lehmer[end - 1] == 0:
        end -= 1
    tokens = [(coeff_order_context(len(lehmer)), end - skip)]
    last = 0
    for v in lehmer[skip:end]:
        tokens.append((coeff_order_context(last), v))
        last = v
    return tokens


def derive(counts_c: np.ndarray, natural, llf: int) -> list[int]:
    """OrderStats::derive (src/coeff_order.rs:586-601): the LLF entries stay,
    the rest by descending count, ties by natural rank."""
    natural = [int(r) for r in natural]
    keys = sorted(((0xFFFFFFFF - int(counts_c[natural[rank]])) << 32) | rank
                  for rank in range(llf, len(natural)))
    return natural[:llf] + [natural[k & 0xFFFFFFFF] for k in keys]


def expected_walk(counts_c: np.ndarray, blocks: int, order, llf: int) -> float:
    """OrderStats::expected_walk (src/coeff_order.rs:570-581), in f64."""
    inv = 1.0 / float(max(blocks, 1))
    none_at_or_after = 1.0
    expected = 0.0
    for raw in reversed([int(r) for r in order[llf:]]):
        expected += 1.0 - none_at_or_after
        p = min(max(float(int(counts_c[raw])) * inv, 0.0), 1.0)
        none_at_or_after *= 1.0 - p
    return expected


def derive_orders(counts, blocks):
    """derive_orders (src/coeff_order.rs:621-673) from the natural orders:
    (used mask, orders[slot][channel] scan position -> raw index, the share of
    the expected walk the adopted orders remove)."""
    used = 0
    orders = [[natural_order(s).tolist() for _ in range(3)] for s in range(len(ORDER_SPECS))]
    natural_walk = saved_walk = 0.0
    for slot, (order_index, llf, _size) in enumerate(ORDER_SPECS):
        nb = int(blocks[slot])
        if nb < MIN_BLOCKS_FOR_ORDER:
            continue
        pos = natural_position(slot)
        derived = [None] * 3
        saved_bits = cost_bits = slot_saved_walk = 0.0
        adopt_any = False
        for c in range(3):
            natural = orders[slot][c]
            cand = derive(counts[slot][c], natural, llf)
            walk = expected_walk(counts[slot][c], nb, natural, llf)
            gain = walk - expected_walk(counts[slot][c], nb, cand, llf)
            natural_walk += walk * float(nb)
            ntokens = len(permutation_tokens([int(pos[r]) for r in cand], llf))
            channel_saved = gain * float(nb) * BITS_PER_SAVED_TOKEN
            channel_cost = float(ntokens) * BITS_PER_PERMUTATION_TOKEN
            if gain > 0.0 and channel_saved > channel_cost * GATE_MARGIN:
                adopt_any = True
                slot_saved_walk += gain * float(nb)
                saved_bits += channel_saved
                cost_bits += channel_cost
                derived[c] = cand
            else:
                derived[c] = natural
        if adopt_any and saved_bits > cost_bits * GATE_MARGIN:
            used |= 1 << order_index
            orders[slot] = derived
            saved_walk += slot_saved_walk
    return used, orders, (saved_walk / natural_walk if natural_walk > 0.0 else 0.0)
