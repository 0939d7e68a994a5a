"""GPU parity: every stage of the CUDA path against the CPU oracle on the
same inputs, through the C ABI.  Integer, index and float results of the
FP32 path are compared bit for bit (the kernels repeat the reference's
arithmetic and summation order with no FMA contraction)."""
import numpy as np
import pytest

from geye_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.int32)


@pytest.fixture(scope="module")
def ctx():
    import geye_gb300 as g
    c = g.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def car(ctx, car_paths):
    import geye_gb300 as g
    return g.Model(ctx, *car_paths), O.Model(*car_paths)


@pytest.fixture(scope="module")
def person(ctx, person_paths):
    import geye_gb300 as g
    return g.Model(ctx, *person_paths), O.Model(*person_paths)


def _img(w, h, seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, size=(3, w, h)).astype(np.float32)
    img[:, : w // 3, : h // 3] = 91.0
    return img


@pytest.mark.parametrize("w,h", [(64, 48), (157, 93), (640, 480)])
def test_resize(ctx, w, h):
    img = _img(w, h, w)
    sc = np.float32(2.0 ** 0.1)
    for ii in (1, 3, 7, 9):
        st = float(np.float32(1.0 / (float(sc) ** ii)))
        assert np.array_equal(bits(ctx.resize(img, st)), bits(O.resize(img, st)))
    assert np.array_equal(bits(ctx.resize(img, 0.5)), bits(O.resize(img, 0.5)))


@pytest.mark.parametrize("sbin", [4, 8])
@pytest.mark.parametrize("w,h", [(64, 48), (131, 99), (640, 480)])
def test_calc_feature(ctx, sbin, w, h):
    img = O.resize(_img(w, h, 3 * w + sbin), 0.91)
    assert np.array_equal(bits(ctx.calc_feature(img, sbin)), bits(O.calc_feature(img, sbin)))


def test_pyramid(ctx, car):
    gm, om = car
    fr = synth.make_frame(640, 480, seed=0)
    gm.reset_scales()
    feats, fs, sc = ctx.calc_f_pyramid(fr, gm)
    P = O.Pyramid(om, fr)
    assert len(feats) == P.LEN == 35
    assert np.array_equal(bits(sc), bits(P.scales))
    for l in range(P.LEN):
        assert tuple(fs[l]) == P.ftsize[l]
        assert np.array_equal(bits(feats[l]), bits(P.feat(l))), f"level {l}"


@pytest.mark.parametrize("shape", [(6, 6), (6, 16), (8, 13), (11, 5)])
def test_fconv(ctx, shape):
    rng = np.random.default_rng(shape[0] * 100 + shape[1])
    feat = rng.random((31, 47, 38)).astype(np.float32) * 0.2
    filt = rng.normal(0, 0.01, size=(31, shape[1], shape[0])).astype(np.float32)
    got = ctx.fconvsMT(feat, [filt, filt * 0.5])
    assert np.array_equal(bits(got[0]), bits(O.fconv(feat, filt)))
    assert np.array_equal(bits(got[1]), bits(O.fconv(feat, filt * 0.5)))


@pytest.mark.parametrize("seed", range(8))
def test_dt(ctx, seed):
    rng = np.random.default_rng(seed)
    d0, d1 = (int(v) for v in rng.integers(1, 200, size=2))
    vals = rng.normal(0, 0.3, size=(d1, d0)).astype(np.float32)
    if seed % 2:
        vals = (np.round(vals * 4) / 4).astype(np.float32)
    lo = 0.001 if seed < 6 else -0.05
    a = rng.uniform(lo, 0.1, size=4).astype(np.float32)
    M, Ix, Iy = ctx.dt(vals, *[float(x) for x in a])
    rM, rIx, rIy = O.dt(vals, *[float(x) for x in a])
    assert np.array_equal(Ix, rIx) and np.array_equal(Iy, rIy)
    assert np.array_equal(bits(M), bits(rM))


def test_model_sym(ctx, tmp_path):
    """rootsym (all 1), part_partner and part_sym as the reference's loader sets them."""
    import geye_gb300 as g
    comp, root, part = synth.write_model_csv(synth.CAR_SPEC, str(tmp_path))
    vals = [v.strip() for v in open(part).read().split(",") if v.strip()]
    n, pos, partners = int(float(vals[0])), 1, []
    for i in range(n):
        h, w, c = (int(float(v)) for v in vals[pos:pos + 3])
        pos += 3 + h * w * c
        partners.append([0, 2, 0, 5][i % 4])
        vals[pos] = f"{partners[-1]:14.6f}"
        pos += 1
    with open(part, "w") as f:
        f.write("".join(v + ",\n" for v in vals))
    m = g.Model(ctx, comp, root, part)
    s = m.sym()
    nor = m.NoR
    m.close()
    assert list(s["rootsym"]) == [1] * nor
    assert list(s["part_partner"]) == partners
    assert list(s["part_sym"]) == [1 if p == 0 else 0 for p in partners]


@pytest.mark.parametrize("seed", range(4))
def test_nms_ties(ctx, seed):
    rng = np.random.default_rng(seed)
    n = [1, 2, 700, 5000][seed]
    GL = 39
    boxes = np.zeros((n, GL), np.float32)
    xy = rng.uniform(0, 600, size=(n, 2)); wh = rng.uniform(10, 150, size=(n, 2))
    boxes[:, 0], boxes[:, 1] = xy[:, 1], xy[:, 0]
    boxes[:, 2], boxes[:, 3] = xy[:, 1] + wh[:, 1], xy[:, 0] + wh[:, 0]
    boxes[:, GL - 2] = np.round(rng.normal(size=n) * 3) / 4
    boxes[:, GL - 1] = np.arange(n)
    keep, _, k = O.nms_keep(boxes, 0.5)
    got = ctx.nms(boxes, 0.5, 8)
    assert got.shape[0] == k
    assert np.array_equal(bits(got), bits(boxes[keep]))


def test_get_boxes_from_oracle_features(ctx, car):
    gm, om = car
    fr = synth.make_frame(320, 240, seed=4)
    P = O.Pyramid(om, fr)
    feats = [P.feat(l) for l in range(P.LEN)]
    S = O.Scores(om, P)
    a_ref = np.full((320, 240), -100, np.float32)
    om.m.im_w, om.m.im_h = 320, 240
    ref, oob = S.boxes(-0.5, a_ref)
    assert oob == 0
    a_gpu = np.full((320, 240), -100, np.float32)
    got = ctx.get_boxes(feats, P.scales, np.array(P.ftsize), gm, -0.5, a_gpu, (320, 240))
    assert got.shape == ref.shape
    assert np.array_equal(bits(got), bits(ref))
    assert np.array_equal(bits(a_gpu), bits(a_ref))


@pytest.mark.parametrize("w,h,seed", [(640, 480, 0), (320, 240, 7)])
def test_car_detection_end_to_end(ctx, car, w, h, seed):
    gm, om = car
    gm.reset_scales()
    om.m.ini = 1
    fr = synth.make_frame(w, h, seed=seed)
    a_gpu = np.full((w, h), -100, np.float32)
    a_ref = np.full((w, h), -100, np.float32)
    got = ctx.car_detection(fr, gm, -0.5, a_gpu, 0.5)
    ref = O.car_detection(om, fr, -0.5, 0.5, a_score=a_ref)
    assert got["num"] == ref["K"] > 0
    assert np.array_equal(got["point"], ref["point"])
    assert np.array_equal(got["or_point"], ref["or_point"])
    assert np.array_equal(got["type"], ref["type"])
    assert np.array_equal(bits(got["score"]), bits(ref["score"]))
    assert np.array_equal(bits(got["scale"]), bits(ref["scale"]))
    assert np.array_equal(bits(a_gpu), bits(a_ref))


def test_car_and_person_1280x720(ctx, car, person):
    (gc, oc), (gp, op) = car, person
    for gm, om in ((gc, oc), (gp, op)):
        gm.reset_scales()
        om.m.ini = 1
    fr = synth.make_frame(1280, 720, seed=1)
    got = ctx.detect_multi(fr, [gc, gp], -0.5, 0.5)
    for res, om in zip(got, (oc, op)):
        ref = O.car_detection(om, fr, -0.5, 0.5)
        assert res["num"] == ref["K"]
        assert np.array_equal(res["point"], ref["point"])
        assert np.array_equal(bits(res["score"]), bits(ref["score"]))


def _all_scores(om, fr):
    S = O.Scores(om, O.Pyramid(om, fr))
    return np.sort(np.concatenate([S.score(l, c).ravel() for l in range(S.interval, S.LEN) if not S.skipped[l]
                                   for c in range(S.NoC)]))[::-1]


@pytest.mark.parametrize("k", [0, 1, 2, 3, 50])
def test_pipeline_few_detections(ctx, car, k):
    """Thresholds that let exactly k root positions through (k = 0: none; 1: the
    reference's NMS never emits a box that is alone at its turn)."""
    gm, om = car
    fr = synth.make_frame(320, 240, seed=9)
    gm.reset_scales()
    om.m.ini = 1
    s = _all_scores(om, fr)
    assert s[k] < s[k - 1] if k else True   # no tie at the cut
    thresh = float(s[k])
    om.m.ini = 1
    ref = O.car_detection(om, fr, thresh, 0.5)
    gm.reset_scales()
    got = ctx.car_detection(fr, gm, thresh, None, 0.5)
    assert got["num"] == ref["K"]
    assert np.array_equal(got["point"], ref["point"])
    assert np.array_equal(bits(got["score"]), bits(ref["score"]))


def test_pipeline_trained_like_models(ctx, tmp_path):
    """Models with the shapes and value statistics of the reference's trained car
    and person models: sparse detections (a few per frame) instead of every
    position, at a threshold that lets some through."""
    import geye_gb300 as g
    fr = synth.make_frame(640, 480, seed=3)
    for spec in (synth.CAR_TRAINED_LIKE, synth.PERSON_TRAINED_LIKE):
        paths = synth.write_model_csv(spec, str(tmp_path))
        om = O.Model(*paths)
        s = _all_scores(om, fr)
        thresh = float(s[min(200, len(s) - 1)])
        om.m.ini = 1
        ref = O.car_detection(om, fr, thresh, 0.5)
        gm = g.Model(ctx, *paths)
        got = ctx.car_detection(fr, gm, thresh, None, 0.5)
        gm.close()
        assert got["num"] == ref["K"] > 0
        assert np.array_equal(got["point"], ref["point"])
        assert np.array_equal(got["type"], ref["type"])
        assert np.array_equal(bits(got["score"]), bits(ref["score"]))


def test_pipeline_flat_deformation(ctx, tmp_path):
    """Deformation weights near zero and of either sign: the DT windows span
    whole lines and the argmin order cannot be proven from the value range, so
    the pipeline takes the checked path (order check, exact replay) with its
    sampled stores."""
    import dataclasses
    import geye_gb300 as g
    spec = dataclasses.replace(synth.CAR_TRAINED_LIKE, name="car_flat", seed=21,
                               def_ranges=((-1e-6, 1e-6), (-0.01, 0.01), (-1e-6, 1e-6), (-0.01, 0.01)))
    fr = synth.make_frame(320, 240, seed=4)
    paths = synth.write_model_csv(spec, str(tmp_path))
    om = O.Model(*paths)
    s = _all_scores(om, fr)
    thresh = float(s[min(100, len(s) - 1)])
    om.m.ini = 1
    ref = O.car_detection(om, fr, thresh, 0.5)
    gm = g.Model(ctx, *paths)
    got = ctx.car_detection(fr, gm, thresh, None, 0.5)
    gm.close()
    assert got["num"] == ref["K"] > 0
    assert np.array_equal(got["point"], ref["point"])
    assert np.array_equal(got["or_point"], ref["or_point"])
    assert np.array_equal(bits(got["score"]), bits(ref["score"]))


@pytest.mark.parametrize("w,h", [(333, 251), (1920, 1080)])
def test_pipeline_odd_and_large_frames(ctx, car, w, h):
    gm, om = car
    gm.reset_scales()
    om.m.ini = 1
    fr = synth.make_frame(w, h, seed=12)
    got = ctx.car_detection(fr, gm, -0.5, None, 0.5)
    ref = O.car_detection(om, fr, -0.5, 0.5)
    assert got["num"] == ref["K"]
    assert np.array_equal(got["point"], ref["point"])
    assert np.array_equal(got["or_point"], ref["or_point"])
    assert np.array_equal(bits(got["score"]), bits(ref["score"]))


def test_nms_sort_levels_adapt_and_fall_back(tmp_path):
    """A plan fits its NMS quicksort levels to the depth its frames need (a
    shallow frame first: few boxes) and returns to the default when a later
    frame needs more (the leftover segments take the exact single-block
    fallback): every result equals a fresh context's, which launches the
    default levels.  (Quicksort order for every model, so that every frame sorts.)"""
    import geye_gb300 as g
    paths = [synth.write_model_csv(s, str(tmp_path)) for s in (synth.CAR_SPEC, synth.PERSON_SPEC)]
    fr = synth.make_frame(640, 480, seed=6)
    c1 = g.Context(0)
    c1.set_nms_order(g.NMS_ORDER_QUICKSORT)
    m1 = [g.Model(c1, *p) for p in paths]
    for thresh in (0.9, 0.9, -0.5, -0.5):
        got = c1.detect_multi(fr, m1, thresh, 0.5)
        c2 = g.Context(0)
        c2.set_nms_order(g.NMS_ORDER_QUICKSORT)
        m2 = [g.Model(c2, *p) for p in paths]
        want = c2.detect_multi(fr, m2, thresh, 0.5)
        for m in m2:
            m.close()
        c2.close()
        for x, y in zip(got, want):
            assert x["num"] == y["num"]
            assert np.array_equal(x["point"], y["point"]) and np.array_equal(x["type"], y["type"])
            assert np.array_equal(bits(x["score"]), bits(y["score"]))
    for m in m1:
        m.close()
    c1.close()


def test_dt_tile_tuning_keeps_results(car_paths, person_paths):
    """After a plan's first frame its DT tile size is timed on that frame's maps
    (1024, 2048 or 4096 outputs per block); later frames use the choice and
    give the first frame's results, bit for bit."""
    import geye_gb300 as g
    fr = synth.make_frame(640, 480, seed=4)
    with g.Context(0) as c:
        ms = [g.Model(c, *p) for p in (car_paths, person_paths)]
        runs = [c.detect_multi(fr, ms, -0.5, 0.5) for _ in range(3)]
        for m in ms:
            t = c.dt_tuning(m)
            assert t["elems"] in (1024, 2048, 4096) and all(x > 0 for x in t["ms"]), t
        for r in runs[1:]:
            for x, y in zip(runs[0], r):
                assert x["num"] == y["num"]
                assert np.array_equal(x["point"], y["point"]) and np.array_equal(bits(x["score"]), bits(y["score"]))
        for m in ms:
            m.close()


def test_model_of_destroyed_context_is_refused(car_paths):
    """A model's filters are freed with the context that loaded it: detecting with
    it afterwards is an argument error on the host, raised before any launch."""
    import geye_gb300 as g
    a = g.Context(0)
    m = g.Model(a, *car_paths)
    a.close()
    frame = np.zeros((48, 64, 3), np.uint8)
    with g.Context(0) as b:
        with pytest.raises(g.GeyeError, match="destroyed"):
            b.car_detection(frame, m)
        with pytest.raises(g.GeyeError, match="destroyed"):
            b.detect_multi(frame, [m])
    m.close()
