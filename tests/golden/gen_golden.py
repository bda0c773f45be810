"""Extract known-answer vectors from the reference's own sources and tests.

Run in the container that holds the reference checkout (it is not available
on the GPU machines):

    python tests/golden/gen_golden.py <path of the reference checkout>

The reference is Rust and cannot be built here, so its golden data are the
constant tables and asserted values that its own unit tests pin:
  - the natural 8x8 coefficient order (src/ac_context.rs K_COEFF_ORDER_8X8,
    checked by `generic_natural_scan_reproduces_the_spec_tables`);
  - the zero-density context tables (src/ac_context.rs:40-53);
  - the high words of the fast_exp2 table (src/adaptive_quant.rs:732-737);
  - quality->distance anchors (src/encode_image.rs:5758-5771);
  - hybrid-uint boundaries and pack_signed values (src/entropy/token.rs tests);
  - dirty_log2f on powers of two (src/adaptive_quant.rs:896-902);
  - the DCT8 band parameters and the static DCT8 dequant table they must
    reproduce within 2e-6 (src/quant_weights.rs:123-128, :246,
    `dct8_matrix_from_bands_matches_static` :3367-3390);
  - the AFV basis (src/afv.rs:48-180, [pixel][vector], the decimal literals
    as written), checked orthonormal by `afv_basis_is_orthonormal` (:413).
The output is tests/golden/reference_tables.json.
"""
from __future__ import annotations

import json
import os
import re
import sys


def _array(src: str, name: str) -> list[int]:
    start = src.index(name)
    body = src[src.index("[", src.index("=", start)) + 1:]
    body = body[: body.index("];")]
    body = re.sub(r"//[^\n]*", "", body)
    return [int(v, 0) for v in re.findall(r"0x[0-9A-Fa-f]+|\d+", body)]


def _floats(src: str, name: str) -> list[float]:
    start = src.index(name)
    body = src[src.index("[", src.index("=", start)) + 1:]
    depth, end = 1, 0
    for i, ch in enumerate(body):
        depth += ch == "["
        depth -= ch == "]"
        if depth == 0:
            end = i
            break
    body = re.sub(r"//[^\n]*", "", body[:end])
    return [float(v) for v in re.findall(r"-?\d+\.\d*(?:e-?\d+)?|-?\d+e-?\d+", body)]


def main(root: str) -> None:
    ac = open(os.path.join(root, "src/ac_context.rs")).read()
    aq = open(os.path.join(root, "src/adaptive_quant.rs")).read()
    order8 = _array(ac, "K_COEFF_ORDER_8X8:")
    freq = _array(ac, "K_COEFF_FREQ_CONTEXT:")
    nonzero = _array(ac, "K_COEFF_NUM_NONZERO_CONTEXT:")
    assert len(order8) == 64 and len(freq) == 64 and len(nonzero) == 64
    exp2 = re.findall(r"\((0x[0-9A-F]+), 0x[0-9A-F]+\)", aq[aq.index("static EXP2FT"):])
    assert len(exp2) == 64
    qw = open(os.path.join(root, "src/quant_weights.rs")).read()
    dct8_bands = _floats(qw, "static DCT8_BANDS:")
    dct8_static = _floats(qw, "static DEQUANT_MATRIX_8X8:")
    assert len(dct8_bands) == 18 and len(dct8_static) == 192, (len(dct8_bands), len(dct8_static))
    afv = open(os.path.join(root, "src/afv.rs")).read()
    afv = afv[afv.index("= [", afv.index("AFV_BASIS_TRANSPOSE:")):]
    afv = afv[: afv.index("];")]
    afv_basis = re.findall(r"-?\d+\.\d+", afv)
    assert len(afv_basis) == 256, len(afv_basis)
    # larger transforms: the library DCT16X8 table as written (decimal
    # literals, parsed to f32 by the compilers), the band parameters of the
    # 16x16 / 32x32 / 16x8 tables, the natural orders and the block-context map
    m16x8 = qw[qw.index("static DEQUANT_MATRIX_16X8:"):]
    m16x8 = m16x8[m16x8.index("= [") + 3:]
    m16x8 = m16x8[: m16x8.index("];")]
    m16x8 = re.findall(r"-?\d+\.\d+(?:e-?\d+)?", re.sub(r"//[^\n]*", "", m16x8))
    assert len(m16x8) == 384, len(m16x8)

    def band_strings(name, n):
        body = qw[qw.index(name):]
        body = body[body.index("= [") + 3:]
        body = body[: body.index("];")]
        vals = re.findall(r"-?\d[\d_]*\.[\d_]*(?:e-?\d+)?", re.sub(r"//[^\n]*", "", body))
        assert len(vals) == 3 * n, (name, len(vals))
        return [v.replace("_", "") for v in vals]

    order16x8 = _array(ac, "K_COEFF_ORDER_16X8:")
    order16x16 = _array(ac, "K_COEFF_ORDER_16X16:")
    order32x32 = _array(ac, "K_COEFF_ORDER_32X32:")
    assert (len(order16x8), len(order16x16), len(order32x32)) == (128, 256, 1024)
    order32x16 = _array(ac, "K_COEFF_ORDER_32X16:")
    assert len(order32x16) == 512
    dgd = open(os.path.join(root, "src/dc_group_data.rs")).read()
    strategy_code_lut = _array(dgd, "STRATEGY_CODE_LUT:")
    assert len(strategy_code_lut) == 24
    strategy_order = _array(ac, "K_STRATEGY_ORDER:")
    block_ctx_map = _array(ac, "K_COMPACT_BLOCK_CONTEXT_MAP:")
    assert len(strategy_order) == 27 and len(block_ctx_map) == 39
    out = {
        "source": "jixel 0.5.14",
        "dequant_matrix_16x8": m16x8,
        "dct16x16_bands": band_strings("static DCT16X16_BANDS:", 7),
        "dct32x32_bands": band_strings("static DCT32X32_BANDS:", 8),
        "dct16x8_bands": band_strings("static DCT16X8_BANDS:", 7),
        "coeff_order_16x8": order16x8,
        "coeff_order_16x16": order16x16,
        "coeff_order_32x32": order32x32,
        "coeff_order_32x16": order32x16,
        "strategy_code_lut": strategy_code_lut,
        "strategy_order": strategy_order,
        "compact_block_context_map": block_ctx_map,
        "afv_basis_transpose": afv_basis,
        "dct8_bands": dct8_bands,
        "dequant_matrix_8x8": dct8_static,
        "coeff_order_8x8": order8,
        # index 0 is the DC slot (0xBAD sentinel in the reference)
        "coeff_freq_context": [None] + freq[1:],
        "coeff_num_nonzero_context": [None] + nonzero[1:],
        "exp2_table_hi_bits": [int(v, 16) for v in exp2],
        "quality_anchors": [[100.0, 0.05], [99.0, 0.1], [90.0, 1.0], [30.0, 6.4],
                            [0.0, 25.0], [-50.0, 25.0], [110.0, 0.05]],
        "quality_anchor_tolerance": 1e-4,
        "quality_25_range": [6.4, 7.0],
        "hybrid_uint": [[16, 16], [17, 16], [20, 17], [31, 19]],
        "pack_signed": [[0, 0], [-1, 1], [1, 2], [-2, 3], [2, 4]],
        "dirty_log2f_pow2_exponents": [-20, 20],
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_tables.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: gen_golden.py <path of the reference checkout>")
    main(sys.argv[1])
