"""Compile the CUDA library in-tree (sm_103a only) with nvcc.

The product is ``jixel_gb300/_build/libjxg.so``: the C ABI of ``include/jxg.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libjxg.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return [os.path.join(CSRC, f) for f in ("jxg_api.cu", "frame_params.cpp")]


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = [
        nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "-shared", "-o", LIB, *sources(), "-I", os.path.join(ROOT, "include"),
    ]
    if extra:
        cmd[1:1] = extra
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
