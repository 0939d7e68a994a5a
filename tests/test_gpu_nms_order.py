"""The whole-path NMS resolves detections in score order (equal scores by input
index) and falls back to the reference's quicksort order (nms.cpp:70-84) for a
model whose kept set could depend on the order among equal scores.  The
synthetic frames' flat rectangles give runs of equal scores at neighbouring
positions; on some frames such a run holds two alive boxes that suppress each
other, and there the plain score order would keep a different set than the
reference (1280x720, seed 3, car model).  Both orders must give the oracle's
kept set, bit for bit."""
import numpy as np
import pytest

from geye_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.int32)


def _same(x, y, where):
    assert x["num"] == y["num"], where
    for k in ("point", "or_point", "type"):
        assert np.array_equal(x[k], y[k]), (where, k)
    for k in ("score", "scale"):
        assert np.array_equal(bits(x[k]), bits(y[k])), (where, k)


@pytest.fixture(scope="module")
def paths(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("nms_order_models"))
    return [synth.write_model_csv(s, d) for s in (synth.CAR_SPEC, synth.PERSON_SPEC)]


# (w, h, seed): frames where the score order alone would do (640x480) and where
# one model needs the quicksort's order (1280x720 seeds 1 and 3: car; seed 2: person)
FRAMES = [(640, 480, 0), (640, 480, 1), (640, 480, 3), (1280, 720, 1), (1280, 720, 2), (1280, 720, 3)]
NEEDS = {(1280, 720, 1): (1, 0), (1280, 720, 2): (0, 1), (1280, 720, 3): (1, 0)}


@pytest.mark.parametrize("conv", ["fp32", "bf16"])
def test_key_order_equals_quicksort_order(paths, conv):
    import geye_gb300 as g
    mode = {"fp32": g.CONV_FP32, "bf16": g.CONV_BF16}[conv]
    ck, cq = g.Context(0, conv=mode), g.Context(0, conv=mode)
    cq.set_nms_order(g.NMS_ORDER_QUICKSORT)
    mk = [g.Model(ck, *p) for p in paths]
    mq = [g.Model(cq, *p) for p in paths]
    for w, h, seed in FRAMES:
        fr = synth.make_frame(w, h, seed=seed)
        got = ck.detect_multi(fr, mk, -0.5, 0.5)
        need = [int(ck.debug_counters(16)[8 * m + 5]) for m in range(2)]
        want = cq.detect_multi(fr, mq, -0.5, 0.5)
        for m, (x, y) in enumerate(zip(got, want)):
            _same(x, y, (w, h, seed, m))
        if conv == "fp32":
            assert tuple(need) == NEEDS.get((w, h, seed), (0, 0)), (w, h, seed, need)
    for m in mk + mq:
        m.close()
    ck.close()
    cq.close()


def test_key_order_fallback_gives_the_oracle_kept_set(paths):
    """1280x720 seed 3: the car model's run of five equal scores at adjacent
    positions (a flat rectangle) holds boxes that suppress each other; the
    quicksort's order among them decides the kept set."""
    import geye_gb300 as g
    fr = synth.make_frame(1280, 720, seed=3)
    om = O.Model(*paths[0])
    ref = O.car_detection(om, fr, -0.5, 0.5)
    with g.Context(0) as c:
        gm = g.Model(c, *paths[0])
        got = c.car_detection(fr, gm, -0.5, None, 0.5)
        assert int(c.debug_counters(8)[5]) == 1
        gm.close()
    assert got["num"] == ref["K"]
    assert np.array_equal(got["point"], ref["point"])
    assert np.array_equal(got["or_point"], ref["or_point"])
    assert np.array_equal(got["type"], ref["type"])
    assert np.array_equal(bits(got["score"]), bits(ref["score"]))
