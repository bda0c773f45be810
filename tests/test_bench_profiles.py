"""The committed ncu summaries parse the way bench.py reads them: every
kernel of the Fastest frame has its DRAM bytes and warp instructions, the
FP32 operation counts sum to the file's stated total, and the counts are
plausible for one 3840x2160 frame."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KERNELS = ["k_xyb", "k_adaptive_quant", "k_tile_quantize", "k_cost_dct8", "k_cost_16x16",
           "k_cost_8x16", "k_cost_16x8", "k_cost_32x32", "k_site", "k_select", "k_retile",
           "k_adjust", "k_mh_incumbent", "k_mh_sum", "k_mh_choose", "k_mh_apply", "k_qf_median",
           "k_layout_dct8", "k_layout_16x16", "k_layout_8x16", "k_layout_16x8", "k_layout_32x32",
           "k_tokenize_layout"]


def _bench():
    spec = importlib.util.spec_from_file_location("_bench_for_tests", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_counters_cover_every_kernel():
    b = _bench()
    for k in KERNELS:
        dram, inst = b.counters_from_profiles(k)
        assert dram is not None and inst is not None, k
        assert 0 <= dram < 2e9 and 0 < inst < 1e9, k


def test_fp32_operations_sum_to_the_stated_total():
    b = _bench()
    ops = b.fp32_ops_from_profiles()
    assert ops is not None and sorted(ops) == sorted(KERNELS)
    stated = [line for line in open(b.FP32_OPS) if line.startswith("# total:")]
    assert len(stated) == 1
    assert sum(ops.values()) == float(stated[0].split()[2])
    # the XYB stage alone: tens of FP32 operations a pixel (the cube root's Halley steps)
    assert 10 * 3840 * 2160 < ops["k_xyb"] < 200 * 3840 * 2160
