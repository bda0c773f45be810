"""Host-side checks of the C ABI that need no GPU."""
import os
import re

import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import _lib
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "jxg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|int64_t|void|float|const char\*)\s+(jxg_\w+)\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = header_functions()
    assert names, "no declarations parsed"
    assert sorted(_lib.EXPORTS) == names
    for n in names:
        assert hasattr(lib, n), n


def test_rust_binding_declares_every_entry_point():
    # the extern "C" block a jixel maintainer would add
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    assert [n for n in header_functions() if f"fn {n}(" not in text] == []


def test_distance_from_quality_matches_oracle():
    for q in np.linspace(-10, 110, 481):
        assert J.distance_from_quality(float(q)) == O.distance_from_quality(float(q)), q


def test_quality_nan_is_rejected():
    with pytest.raises(J.EncodeError) as e:
        J.distance_from_quality(float("nan"))
    assert e.value.variant == "QualityIsNaN"


def test_frame_info_matches_image_dim():
    fi = J.frame_info(3840, 2160)
    assert (fi.xsize_blocks, fi.ysize_blocks) == (480, 270)
    assert (fi.xsize_groups, fi.ysize_groups, fi.num_groups) == (15, 9, 135)
    assert fi.num_dc_groups == 4
    assert (fi.xsize_tiles, fi.ysize_tiles) == (60, 34)
    fi = J.frame_info(1, 1)
    assert (fi.xsize_blocks, fi.num_groups, fi.num_dc_groups) == (1, 1, 1)


@pytest.mark.parametrize("args,variant", [
    ((0, 5, 3, 8), "EmptyImage"),
    ((5, 0, 3, 8), "EmptyImage"),
    ((1 << 30, 1, 3, 8), "DimensionTooLarge"),
    ((8, 8, 5, 8), "BadChannelCount"),
    ((8, 8, 3, 11), "BadBitDepth"),
])
def test_input_validation(args, variant):
    cfg = J.EncodeConfig(distance=1.0, speed=J.Speed.ULTRA_FAST)
    with pytest.raises(J.EncodeError) as e:
        J.api.validate_input(*args, cfg)
    assert e.value.variant == variant


@pytest.mark.parametrize("d", [0.0, -1.0, float("inf"), float("nan")])
def test_invalid_distance(d):
    cfg = J.EncodeConfig(distance=d, speed=J.Speed.ULTRA_FAST)
    with pytest.raises(J.EncodeError) as e:
        J.api.validate_input(8, 8, 3, 8, cfg)
    assert e.value.variant == "InvalidDistance"


def test_unbuilt_speed_tiers_are_unsupported():
    for s in (J.Speed.FAST, J.Speed.SLOW):
        with pytest.raises(J.EncodeError) as e:
            J.api.validate_input(8, 8, 3, 8, J.EncodeConfig(distance=1.0, speed=s))
        assert e.value.variant == "Unsupported"
    J.api.validate_input(8, 8, 3, 8, J.EncodeConfig(distance=1.0, speed=J.Speed.ULTRA_FAST))


def test_transfer_and_depth_validation():
    # the H.273 codes select_transfer takes; PQ and HLG need the display
    # model, which is not built; 9-bit samples are no entry point's
    TF = J.TransferFunction
    ok = J.EncodeConfig(distance=1.0, speed=J.Speed.ULTRA_FAST)
    for bits in (8, 10, 12, 16):
        for tf in (TF.SRGB, TF.LINEAR, TF.BT709, TF.BT470M, TF.BT470BG, TF.SMPTE240, TF.SMPTE428,
                   TF.UNSPECIFIED, TF.BT2020_12BIT):
            J.api.validate_input(8, 8, 3, bits, ok.with_transfer(tf))
    for tf in (TF.SMPTE2084, TF.HLG):
        with pytest.raises(J.EncodeError) as e:
            J.api.validate_input(8, 8, 3, 16, ok.with_transfer(tf))
        assert e.value.variant == "Unsupported"
    bad = J.EncodeConfig(distance=1.0, speed=J.Speed.ULTRA_FAST)
    bad.transfer = 3  # reserved code
    with pytest.raises(J.EncodeError) as e:
        J.api.validate_input(8, 8, 3, 8, bad)
    assert e.value.variant == "InvalidArgument"
    with pytest.raises(J.EncodeError) as e:
        J.api.validate_input(8, 8, 3, 9, J.EncodeConfig(distance=1.0, speed=J.Speed.ULTRA_FAST))
    assert e.value.variant == "BadBitDepth"
