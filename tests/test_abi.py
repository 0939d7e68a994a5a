"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, exports
every entry point include/geye_dpm.h declares, and fails with a status code
(never a crash or a CPU fallback) when no usable GPU is present."""
import ctypes as C

import numpy as np
import pytest

import geye_gb300 as g
from geye_gb300 import dpm


def test_library_exports_every_declared_symbol():
    L = g.lib()
    declared = dpm.symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_version_and_sm103a_build():
    assert b"sm_103a" in g.lib().geye_version()


def test_null_arguments_are_rejected():
    L = g.lib()
    assert L.geye_ctx_create(0, None, None) == 1                    # GEYE_ERR_ARG
    assert L.geye_nms(None, None, 0.5, None, 8, None) == 1
    assert L.geye_model_info(None, None) == 1
    assert L.geye_ctx_destroy(None) == 0
    assert L.geye_result_free(None) == 0


def test_no_gpu_fails_loudly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(g.GeyeError):
        g.Context(0)
