"""geye_gb300: CPFL/geye's DPM detection path on GB300 (sm_103a).

The product is libgeye_dpm.so (C ABI in include/geye_dpm.h, CUDA kernels and a
C++ host runtime under geye_gb300/csrc).  This package builds it
(geye_gb300.build), wraps it for Python callers (geye_gb300.dpm) and generates
seeded synthetic frames and models (geye_gb300.synth).

Importing the package asks CUDA for 32 hardware work queues
(CUDA_DEVICE_MAX_CONNECTIONS, unless the environment sets it; CUDA reads it
when the process's first context is created, so import this package, or set
the variable, before other CUDA work): a server keeps frames of many slots in flight on separate
streams, and with the default 8 queues those streams share queues and wait on
one another (16 slots at 640x480: 2954 against 3384 frames/s end to end).
"""
import os as _os

_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import build, synth  # noqa: F401,E402
from .dpm import (CONV_BF16, CONV_FP8, CONV_FP32, NMS_ORDER_KEY, NMS_ORDER_QUICKSORT, Batch, Context,  # noqa: F401
                  GeyeError, Model, Server, lib)
