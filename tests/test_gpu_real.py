"""The FP32 drop-in on the reference's own test data: its trained car and
person models on its 21 test frames (tests/golden/real_*.npz), at the
reference's run parameters (thresh -0.5, overlap 0.4).  Detections, the
A_SCORE map and every (level, component) score map are bit-identical to the
oracle's, through the whole path and through the reference's stage
decomposition (calc_f_pyramid -> get_boxes -> nms -> get_new_rects).  The
BF16 and FP8 tensor-core paths report their detection agreement with FP32 on
the same frames."""
import json
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import real_data as RD  # noqa: E402

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def frames():
    return RD.load_frames()


@pytest.fixture(scope="module")
def model_paths(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("real_models"))
    return {n: RD.write_model_csv(RD.model_dump(n), d, n) for n in RD.MODEL_NAMES}


@pytest.fixture(scope="module")
def ctx():
    import geye_gb300 as g
    c = g.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def models(ctx, model_paths):
    import geye_gb300 as g
    ms = {n: g.Model(ctx, *model_paths[n], RD.RATIO) for n in RD.MODEL_NAMES}
    yield ms
    for m in ms.values():
        m.close()


def _check_result(res, E, where):
    assert res["num"] == len(E["score"]), (where, res["num"], len(E["score"]))
    for k in ("point", "or_point", "type"):
        assert np.array_equal(res[k], E[k]), (where, k)
    for k in ("scale", "score"):
        assert np.array_equal(bits(res[k]), bits(E[k])), (where, k)


def test_loader_fields_of_the_trained_models(models):
    """geye_model_load_csv against the reference loader's parse (load_model.cpp:57-530)."""
    for name, m in models.items():
        f = RD.parse_dump(RD.model_dump(name))
        info = m.info()
        assert info["numcomponent"] == f["numcomponent"] and info["sbin"] == f["sbin"]
        assert info["interval"] == f["interval"] and info["numpart0"] == f["comps"][0]["numpart"]
        assert info["NoR"] == len(f["roots"]) and info["NoP"] == len(f["parts"])
        sym = m.sym()
        assert list(sym["rootsym"]) == [r["sym"] for r in f["roots"]]
        assert list(sym["part_partner"]) == [p["partner"] for p in f["parts"]]
        assert list(sym["part_sym"]) == [p["sym"] for p in f["parts"]]


@pytest.mark.parametrize("name", RD.MODEL_NAMES)
def test_fp32_whole_path_bit_identical_on_all_frames(ctx, models, frames, name):
    m = models[name]
    for i in range(RD.N_FRAMES):
        E = RD.expected(name, i)
        a = np.full((640, 480), -100, np.float32)
        res = ctx.car_detection(frames[i], m, RD.THRESH, a, RD.OVERLAP)
        _check_result(res, E, (name, i))
        assert RD.float_digest(a) == E["a_score_sha256"].tobytes(), (name, i, "A_SCORE")
        for (lv, c), want in zip(E["score_maps"], E["score_sha256"]):
            got = ctx.score_map(m, int(lv), int(c))
            assert RD.float_digest(got) == want.tobytes(), (name, i, "score map", int(lv), int(c))


@pytest.mark.parametrize("name", RD.MODEL_NAMES)
def test_fp32_stage_decomposition_on_all_frames(ctx, models, frames, name):
    """calc_f_pyramid -> get_boxes -> nms -> get_new_rects, as detect() and car_detection() chain them."""
    m = models[name]
    for i in range(RD.N_FRAMES):
        E = RD.expected(name, i)
        feats, fs, sc = ctx.calc_f_pyramid(frames[i], m)
        a = np.full((640, 480), -100, np.float32)
        boxes = ctx.get_boxes(feats, sc, fs, m, RD.THRESH, a, img_size=(640, 480))
        assert boxes.shape[0] == int(E["D"]), (name, i)
        kept = ctx.nms(boxes, RD.OVERLAP, m.info()["numpart0"])
        assert np.array_equal(bits(kept), bits(E["kept"])), (name, i)
        _check_result(ctx.get_new_rects((640, 480), m, kept), E, (name, i, "get_new_rects"))
        assert RD.float_digest(a) == E["a_score_sha256"].tobytes(), (name, i, "A_SCORE")


def test_fp32_both_models_in_one_call(ctx, models, frames):
    """detect_multi shares one pyramid between the models; each model's result is its own call's."""
    ms = [models[n] for n in RD.MODEL_NAMES]
    for i in (0, 4, 13, 20):
        a_s = [np.full((640, 480), -100, np.float32) for _ in ms]
        res = ctx.detect_multi(frames[i], ms, RD.THRESH, RD.OVERLAP, a_s)
        for name, r, a in zip(RD.MODEL_NAMES, res, a_s):
            E = RD.expected(name, i)
            _check_result(r, E, (name, i, "multi"))
            assert RD.float_digest(a) == E["a_score_sha256"].tobytes(), (name, i)


def _iou(a, b):
    w = min(a[2], b[2]) - max(a[0], b[0]) + 1
    h = min(a[3], b[3]) - max(a[1], b[1]) + 1
    inter = max(0, w) * max(0, h)
    ua = (a[2] - a[0] + 1) * (a[3] - a[1] + 1) + (b[2] - b[0] + 1) * (b[3] - b[1] + 1) - inter
    return inter / ua if ua > 0 else 0.0


def test_tensor_core_modes_agree_on_real_frames(model_paths, frames):
    import geye_gb300 as g
    report = {}
    for mode_name, mode in (("bf16", g.CONV_BF16), ("fp8", g.CONV_FP8)):
        with g.Context(0, conv=mode) as c:
            ms = [g.Model(c, *model_paths[n], RD.RATIO) for n in RD.MODEL_NAMES]
            n = hit = 0
            for i in range(RD.N_FRAMES):
                res = c.detect_multi(frames[i], ms, RD.THRESH, RD.OVERLAP)
                for name, r in zip(RD.MODEL_NAMES, res):
                    E = RD.expected(name, i)
                    for p, t in zip(E["point"], E["type"]):
                        n += 1
                        hit += any(r["type"][j] == t and _iou(p, r["point"][j]) >= 0.9 for j in range(r["num"]))
            for m in ms:
                m.close()
        report[mode_name] = {"fp32_detections": n, "matched": hit, "agreement": hit / max(n, 1)}
    out = os.environ.get("GEYE_REAL_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)
    print(report)
    assert report["bf16"]["agreement"] >= 0.9, report


@pytest.mark.parametrize("name", RD.MODEL_NAMES)
def test_get_new_rects_against_the_reference_function(ctx, model_paths, name):
    """geye_get_new_rects on the records the reference's own get_new_rects
    (tracking.cpp:90-166) regressed: every kept record, and those records moved
    past each image border, at two model ratios; bit for bit."""
    import geye_gb300 as g
    boxes, want = RD.get_new_rects_vectors(name)
    for ratio in RD.GNR_RATIOS:
        m = g.Model(ctx, *model_paths[name], ratio)
        _check_result(ctx.get_new_rects((640, 480), m, boxes), want[ratio], (name, ratio))
        m.close()
