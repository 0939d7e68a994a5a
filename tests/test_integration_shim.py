"""INTEGRATION.md's reference-side shim compiles against the reference's own
prototype headers (CAR_TRACKING/car_det_func.h, detect_func.h,
get_boxes_func.h, for_use_GPU.h, MODEL_info.h) and include/geye_dpm.h.

-Werror=missing-declarations turns a shim definition whose signature no longer
matches the reference's declaration (C++ would take it as a new overload) into
an error, and a geye_* call that no longer matches the C ABI fails to compile:
a signature that drifts on either side breaks this test.  Runs where the
reference's sources are present (the OpenCV stand-in headers of oracle/ref/shim
supply IplImage)."""
import os
import re
import shutil
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _shim_source() -> str:
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", doc, flags=re.S)
    src = [b for b in blocks if b.startswith("// geye_shim.cpp")]
    assert len(src) == 1, "INTEGRATION.md must hold exactly one geye_shim.cpp block"
    return src[0]


def test_shim_block_names_every_replaced_entry_point():
    src = _shim_source()
    for name in ("init_cuda", "clean_cuda", "car_detection", "calc_f_pyramid", "get_boxes", "nms", "get_new_rects",
                 "dt", "resize", "calc_feature", "flip_feat"):
        assert re.search(rf"\b{name}\(", src), name


@pytest.mark.skipif(not os.path.isdir(O.REF_SRC_DIR), reason="reference sources not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_shim_compiles_against_reference_headers_and_the_c_abi(tmp_path):
    src = tmp_path / "geye_shim.cpp"
    src.write_text(_shim_source())
    cmd = ["g++", "-std=c++17", "-c", "-o", str(tmp_path / "geye_shim.o"), "-Wall", "-Werror=missing-declarations",
           "-Wno-unused-function", "-Wno-unused-variable", "-Wno-write-strings",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle", "ref", "shim"),
           "-I", O.REF_SRC_DIR, "-I", "/usr/local/cuda/include", str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    # every geye_* symbol the shim uses is one the library exports (declared in the header)
    from geye_gb300 import dpm
    used = set(re.findall(r"\b(geye_[a-z_]+)\(", src.read_text()))
    assert used <= set(dpm.symbols()), used - set(dpm.symbols())
