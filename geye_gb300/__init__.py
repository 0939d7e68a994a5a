"""geye_gb300: CPFL/geye's DPM detection path on GB300 (sm_103a).

The product is libgeye_dpm.so (C ABI in include/geye_dpm.h, CUDA kernels and a
C++ host runtime under geye_gb300/csrc).  This package builds it
(geye_gb300.build), wraps it for Python callers (geye_gb300.dpm) and generates
seeded synthetic frames and models (geye_gb300.synth).
"""
from . import build, synth  # noqa: F401
from .dpm import (CONV_BF16, CONV_FP8, CONV_FP32, NMS_ORDER_KEY, NMS_ORDER_QUICKSORT, Batch, Context,  # noqa: F401
                  GeyeError, Model, Server, lib)
