"""Pins the CPU oracle to the reference's own outputs recorded in
tests/golden/ref_vectors.npz (written by tests/golden/make_golden.py from the
reference's CPU functions).  Runs everywhere, including machines without the
reference sources; tests/test_oracle_vs_ref.py repeats the comparison live
where the sources are present."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_vectors.npz")


@pytest.fixture(scope="module")
def V():
    return np.load(GOLD)


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.int32) if a.dtype == np.float32 else a,
                                                 b.view(np.int32) if b.dtype == np.float32 else b)


def test_resize(V):
    for k, s in enumerate(V["resize_scales"]):
        assert _same(O.resize(V["resize_in"], float(s)), V[f"resize_out{k}"]), f"scale {s}"


def test_calc_feature(V):
    for sbin in (4, 8):
        assert _same(O.calc_feature(V["feat_in"], sbin), V[f"feat_out{sbin}"]), f"sbin {sbin}"


def test_flip_feat(V):
    assert _same(O.flip_feat(V["flip_in"]), V["flip_out"])


def test_dt(V):
    for k in range(4):
        M, Ix, Iy = O.dt(V[f"dt_in{k}"], *[float(c) for c in V[f"dt_coef{k}"]])
        assert _same(M, V[f"dt_M{k}"]) and _same(Ix, V[f"dt_Ix{k}"]) and _same(Iy, V[f"dt_Iy{k}"]), f"case {k}"


def test_quicksort_and_nms(V):
    for k in range(3):
        a, order = O.quicksort(V[f"qs_in{k}"])
        assert _same(a, V[f"qs_val{k}"]) and _same(order, V[f"qs_ord{k}"]), f"case {k}"
        keep, _, _ = O.nms_keep(V[f"nms_in{k}"], 0.5)
        assert np.array_equal(keep, V[f"nms_keep{k}"].astype(bool)), f"case {k}"


def test_add_part_and_boxes(V):
    score, M = V["ap_score"], V["ap_M"]
    r1, r0 = score.shape
    p1, p0 = M.shape
    for k, (ax, ay) in enumerate(V["ap_anchor"]):
        s = score.copy()
        O.lib().orc_add_part(O._ptr(s), O._ptr(O._f32(M)), O._ptr(O._i32([r0, r1])), O._ptr(O._i32([p0, p1])),
                             int(ax), int(ay))
        assert _same(s, V[f"ap_out{k}"])
    Ix, Iy = V["pb_Ix"], V["pb_Iy"]
    for i, s in enumerate(V["box_scales"]):
        for j, (x, y) in enumerate(V["box_pts"]):
            a = np.zeros(4, np.float32)
            O.lib().orc_rootbox(int(x), int(y), float(s), 0, 0, O._ptr(O._i32([6, 16])), O._ptr(a))
            assert _same(a, V["rootbox_out"][i, j])
            a = np.zeros(4, np.float32)
            O.lib().orc_partbox(int(x), int(y), 3, 2, float(s), 0, 0, O._ptr(O._i32([6, 6])), O._ptr(O._i32(Ix)),
                                O._ptr(O._i32(Iy)), O._ptr(O._i32([Ix.shape[1], Ix.shape[0]])), O._ptr(a))
            assert _same(a, V["partbox_out"][i, j])


def test_calc_a_score_and_gmpc(V):
    score = V["as_score"]
    s1, s0 = score.shape
    for k, s in enumerate(V["as_scales"]):
        a = np.full((160, 120), -100, np.float32)
        O.lib().orc_calc_a_score(O._ptr(a), O._ptr(score), O._ptr(O._i32([s0, s1])), O._ptr(O._i32([6, 16])),
                                 120, 160, 0, 0, float(s))
        assert _same(a, V[f"as_out{k}"])
    ys, xs = np.nonzero(score.T > np.float32(0.3))   # get_gmpc's column-major scan: x outer, y inner
    order = np.lexsort((ys, xs))
    assert np.array_equal(np.stack([ys[order], xs[order]], 1), V["gmpc_out"])


def test_max_scale(V, car_paths, person_paths):
    for paths, key in ((car_paths, "ms_car"), (person_paths, "ms_person")):
        m = O.Model(*paths)
        for (w, h), want in zip(V["ms_sizes"], V[key]):
            assert m.max_scale(int(w), int(h)) == want
