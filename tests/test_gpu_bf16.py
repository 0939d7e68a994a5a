"""The tensor-core (tcgen05, BF16 operands, FP32 accumulation) convolution.

BF16 keeps 8 significant bits, so rounding a feature and a filter value each
costs at most a relative 2**-8 / 2; products are exact and the FP32 sums add
far less, so every map value is within 2**-7 * sum|a*b| of the FP32 result
(checked with a 5% margin).  Inputs whose values are exact in BF16 and whose
partial sums are exact in FP32 must give bit-identical maps: that case pins
the operand layouts (any wrong tap, channel or row shows up).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx16():
    import geye_gb300 as g
    c = g.Context(0, conv=g.CONV_BF16)
    yield c
    c.close()


def _maps_within_bound(got, feat, filters):
    for m, f in zip(got, filters):
        ref = O.fconv(feat, f)
        mag = O.fconv(np.abs(feat), np.abs(f))
        err = np.abs(m.astype(np.float64) - ref.astype(np.float64))
        assert np.all(err <= 1.05 * 2.0 ** -7 * mag + 1e-7), float((err / (mag + 1e-12)).max())


def test_bf16_exact_values_are_bit_identical(ctx16):
    rng = np.random.default_rng(3)
    feat = (rng.integers(0, 5, size=(31, 41, 37)) * 0.25).astype(np.float32)
    shapes = [(6, 6), (6, 6), (6, 16), (8, 13), (11, 5)]
    filters = [rng.integers(-2, 3, size=(31, b1, b0)).astype(np.float32) for b0, b1 in shapes]
    got = ctx16.fconvsMT(feat, filters)
    for m, f in zip(got, filters):
        assert np.array_equal(m, O.fconv(feat, f))


@pytest.mark.parametrize("nparts", [1, 16, 24])
def test_bf16_maps_within_rounding_bound(ctx16, nparts):
    rng = np.random.default_rng(nparts)
    feat = (rng.random((31, 78, 58)) * 0.4).astype(np.float32)
    filters = [rng.normal(0, 0.01, size=(31, 6, 6)).astype(np.float32) for _ in range(nparts)]
    filters += [rng.normal(0, 0.01, size=(31, 16, 6)).astype(np.float32)]
    _maps_within_bound(ctx16.fconvsMT(feat, filters), feat, filters)


def test_bf16_large_map_many_ctas(ctx16):
    # a 1280x720 level-0 sized map: several CTAs per filter group, slabs near the plane end
    rng = np.random.default_rng(7)
    feat = (rng.random((31, 318, 178)) * 0.4).astype(np.float32)
    filters = [rng.normal(0, 0.01, size=(31, 6, 6)).astype(np.float32) for _ in range(24)]
    _maps_within_bound(ctx16.fconvsMT(feat, filters), feat, filters)


def _iou(a, b):
    x1, y1 = max(a[0], b[0]), max(a[1], b[1])
    x2, y2 = min(a[2], b[2]), min(a[3], b[3])
    inter = max(0, x2 - x1 + 1) * max(0, y2 - y1 + 1)
    ua = (a[2] - a[0] + 1) * (a[3] - a[1] + 1) + (b[2] - b[0] + 1) * (b[3] - b[1] + 1) - inter
    return inter / ua if ua > 0 else 0.0


def agreement(ref, got):
    """Share of reference detections with a same-component match of IoU >= 0.9."""
    n = ref["num"]
    if n == 0:
        return 1.0 if got["num"] == 0 else 0.0
    hit = 0
    for i in range(n):
        for j in range(got["num"]):
            if got["type"][j] == ref["type"][i] and _iou(ref["point"][i], got["point"][j]) >= 0.9:
                hit += 1
                break
    return hit / n


def test_bf16_pipeline_detection_agreement(tmp_path):
    import geye_gb300 as g
    from geye_gb300 import synth
    frame = synth.make_frame(640, 480, seed=0)
    res = {}
    for mode in (g.CONV_FP32, g.CONV_BF16):
        with g.Context(0, conv=mode) as c:
            ms = [g.Model(c, *synth.write_model_csv(s, str(tmp_path))) for s in (synth.CAR_SPEC, synth.PERSON_SPEC)]
            res[mode] = c.detect_multi(frame, ms, -0.5, 0.5, None)
            for m in ms:
                m.close()
    for r32, r16 in zip(res[g.CONV_FP32], res[g.CONV_BF16]):
        assert r32["num"] > 0
        assert agreement(r32, r16) >= 0.9


def test_bf16_filter_columns_in_phases(ctx16):
    # 16 filter columns over 320-row levels: bank and slab of the whole filter do not fit in shared
    # memory at once, so the kernel walks the filter columns in phases, accumulating in TMEM
    rng = np.random.default_rng(11)
    feat = (rng.integers(0, 5, size=(31, 60, 320)) * 0.25).astype(np.float32)
    filters = [rng.integers(-2, 3, size=(31, 16, 6)).astype(np.float32) for _ in range(3)]
    got = ctx16.fconvsMT(feat, filters)
    for m, f in zip(got, filters):
        assert np.array_equal(m, O.fconv(feat, f))


def test_conv_tile_shape_autotuner(tmp_path):
    import geye_gb300 as g
    from geye_gb300 import synth
    frame = synth.make_frame(640, 480, seed=2)
    with g.Context(0, conv=g.CONV_BF16) as c:
        ms = [g.Model(c, *synth.write_model_csv(s, str(tmp_path))) for s in (synth.CAR_SPEC, synth.PERSON_SPEC)]
        c.detect_multi(frame, ms, -0.5, 0.5, None)
        tuned = [c.conv_tuning(m) for m in ms]
        for m in ms:
            m.close()
    assert tuned[0] == tuned[1]   # one launch convolves both models
    for t in tuned:
        assert t["tiles_per_cta"] in (0, 1, 2, 4, 8)   # 0: the persistent form (one CTA per SM)
        assert 64 <= t["smem_kb"] <= 227 and t["ctas"] > 0 and t["ms"] > 0


@pytest.mark.parametrize("mode", ["bf16", "fp8"])
@pytest.mark.parametrize("w,h", [(320, 240), (640, 480), (1280, 720)])
def test_conv_persistent_form_matches_stage_ring(tmp_path, monkeypatch, mode, w, h):
    """The persistent form (bank resident, one CTA per SM) runs every tile's MMAs in
    the stage-ring form's order: same detections and scores, bit for bit."""
    import geye_gb300 as g
    from geye_gb300 import synth
    conv = {"bf16": g.CONV_BF16, "fp8": g.CONV_FP8}[mode]
    paths = [synth.write_model_csv(s, str(tmp_path)) for s in (synth.CAR_SPEC, synth.PERSON_SPEC)]
    frame = synth.make_frame(w, h, seed=7)
    out = {}
    for shape in ("0", "10"):
        monkeypatch.setenv("GEYE_TC_SHAPE", shape)
        with g.Context(0, conv=conv) as c:
            ms = [g.Model(c, *p) for p in paths]
            out[shape] = (c.detect_multi(frame, ms, -0.5, 0.5), c.conv_tuning(ms[0]))
            for m in ms:
                m.close()
    (ring, t_ring), (pers, t_pers) = out["0"], out["10"]
    assert t_ring["tiles_per_cta"] == 4 and t_pers["tiles_per_cta"] == 0
    for a, b in zip(ring, pers):
        assert a["num"] == b["num"]
        for k in ("point", "or_point", "type"):
            assert np.array_equal(a[k], b[k])
        for k in ("score", "scale"):
            assert np.array_equal(np.asarray(a[k], np.float32).view(np.int32), np.asarray(b[k], np.float32).view(np.int32))


@pytest.mark.parametrize("n", [40, 64])
def test_bf16_wide_filter_groups_bit_identical(ctx16, n):
    """Groups of up to 64 filters (MMA N = 48, 64): exact-valued inputs give the FP32 maps bit for bit."""
    rng = np.random.default_rng(n)
    feat = (rng.integers(0, 5, size=(31, 30, 26)) * 0.25).astype(np.float32)
    filters = [rng.integers(-2, 3, size=(31, 6, 6)).astype(np.float32) for _ in range(n)]
    got = ctx16.fconvsMT(feat, filters)
    for m, f in zip(got, filters):
        assert np.array_equal(m.view(np.int32), O.fconv(feat, f).view(np.int32))


def test_bf16_root_blocks_on_split_operands(tmp_path):
    """Root filters in the pipeline run as blocks of the part grid on split BF16
    operands (hi*hi + hi*lo + lo*hi).  With every part filter zero (their maps and
    DT outputs are then exactly equal in both modes), a score map differs from the
    FP32 pipeline's only by its root: within 2**-14 * sum|a*b| of the FP32 root,
    128 times tighter than plain BF16 operands allow, so a wrong block, tap,
    shift or remainder plane shows at once."""
    import geye_gb300 as g
    from geye_gb300 import synth
    spec = synth.ModelSpec("car_zp", roots=[(6, 16), (8, 13)], seed=31,
                           parts=[[(6, 6)] * 4, [(6, 6)] * 4], root_std=0.01, part_std=0.0,
                           offsets=[0.05, -0.03], def_ranges=((0.01, 0.1),) * 4)
    paths = synth.write_model_csv(spec, str(tmp_path))
    frame = synth.make_frame(640, 480, seed=5)
    om = O.Model(*paths)
    S = O.Scores(om, O.Pyramid(om, frame))
    maps = {}
    for mode in (g.CONV_FP32, g.CONV_BF16):
        with g.Context(0, conv=mode) as c:
            m = g.Model(c, *paths)
            c.detect_multi(frame, [m], -0.5, 0.5, None)
            maps[mode] = {(lv, k): c.score_map(m, lv, k) for lv in range(S.interval, S.LEN) if not S.skipped[lv]
                          for k in range(S.NoC)}
            m.close()
    worst = 0.0
    for key, s32 in maps[g.CONV_FP32].items():
        s64, mag = S.score_f64(*key)
        err = np.abs(maps[g.CONV_BF16][key].astype(np.float64) - s32.astype(np.float64)).max()
        worst = max(worst, err / mag)
        assert err <= 2.0 ** -14 * mag, (key, err, mag)
    assert worst > 0   # the split path ran (plain FP32 would give exactly 0)
