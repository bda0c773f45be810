"""Write the decoder-shared constant tables of the larger transforms as C.

The JPEG XL library's default DCT16X8 / DCT8X16 dequantisation weights, and
the band parameters of the DCT16X16, DCT32X32 and DCT16X8 tables, are what a
decoder applies when a frame signals no custom table, so the encoder must
quantise with the same f32 values.  They are kept as the decimal literals the
reference writes (src/quant_weights.rs:455-1013): both C compilers round a
decimal literal with the `f` suffix to the nearest f32, as Rust does.

Input: tests/golden/reference_tables.json (extracted from the reference's
sources by tests/golden/gen_golden.py).  Output: library_tables.h beside this
script (the CUDA library's host code) and oracle/library_tables.inc (the
oracle).  Run once after regenerating the JSON:

    python jixel_gb300/csrc/gen_library_tables.py
"""
from __future__ import annotations

import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _literal(s: str) -> str:
    return s + ("f" if ("." in s or "e" in s) else ".0f")


def _rows(values: list[str], per_row: int, indent: str) -> str:
    lines = []
    for i in range(0, len(values), per_row):
        lines.append(indent + ", ".join(_literal(v) for v in values[i:i + per_row]) + ",")
    return "\n".join(lines)


def _table(ctype: str, name: str, values: list[str], rows: int, cols: int) -> str:
    assert len(values) == rows * cols
    out = [f"static const {ctype} {name}[{rows}][{cols}] = {{"]
    for r in range(rows):
        out.append("    {")
        out.append(_rows(values[r * cols:(r + 1) * cols], 6, "        "))
        out.append("    },")
    out.append("};")
    return "\n".join(out)


def main() -> None:
    d = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_tables.json")))
    body = "\n\n".join([
        "/* DCT16X16 band parameters (X, Y, B; src/quant_weights.rs:927-961) */\n"
        + _table("float", "LIB_DCT16X16_BANDS", d["dct16x16_bands"], 3, 7),
        "/* DCT32X32 band parameters (src/quant_weights.rs:963-1000) */\n"
        + _table("float", "LIB_DCT32X32_BANDS", d["dct32x32_bands"], 3, 8),
        "/* DCT16X8 band parameters (src/quant_weights.rs:1006-1013) */\n"
        + _table("float", "LIB_DCT16X8_BANDS", d["dct16x8_bands"], 3, 7),
        "/* library DCT16X8 / DCT8X16 weights, flat coefficient index\n"
        " * (src/quant_weights.rs:455-925) */\n"
        + _table("float", "LIB_DCT16X8_MATRIX", d["dequant_matrix_16x8"], 3, 128),
    ])
    head = ("Generated by jixel_gb300/csrc/gen_library_tables.py from the reference's "
            "constant tables;\n * do not edit.")
    with open(os.path.join(HERE, "library_tables.h"), "w") as fh:
        fh.write(f"// {head.replace(chr(10) + ' *', chr(10) + '//')}\n#pragma once\n\n"
                 "namespace jxg {\n\n" + body + "\n\n}  // namespace jxg\n")
    with open(os.path.join(ROOT, "oracle", "library_tables.inc"), "w") as fh:
        fh.write(f"/* {head} */\n\n" + body + "\n")
    print("wrote library_tables.h and oracle/library_tables.inc")


if __name__ == "__main__":
    main()
