"""GB300-native VarDCT front end with jixel's encoder interface.

The compute runs in the CUDA library ``_build/libjxg.so`` (C ABI in
``include/jxg.h``); this package is its host-side mirror.
"""
from .api import (EncodeConfig, EncodeError, FrontendBatch, FrontendContext, FrontendResult,
                  PinnedOutputs, Speed, TransferFunction, ac_bits_estimate, derive_orders,
                  distance_from_quality, encode_frontend, frame_info)

__all__ = [
    "EncodeConfig", "EncodeError", "FrontendBatch", "FrontendContext", "FrontendResult", "Speed",
    "PinnedOutputs", "TransferFunction", "ac_bits_estimate", "derive_orders", "distance_from_quality",
    "encode_frontend", "frame_info",
]
