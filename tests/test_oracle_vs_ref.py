"""Pins the CPU oracle (oracle/dpm_oracle.c) to the reference's own CPU
functions compiled from the reference sources (oracle/_ref).  Runs only where
the reference sources are present; elsewhere tests/test_golden.py pins the
oracle through the committed vectors these functions produced."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.skipif(O.ref_lib() is None, reason="reference sources not present to build oracle/_ref")


def _img(w, h, seed, flat_frac=0.3):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, size=(3, w, h)).astype(np.float32)
    # flat patches produce exact ties and zero gradients, as the synthetic frames do
    fw, fh = int(w * flat_frac), int(h * flat_frac)
    img[:, :fw, :fh] = 77.0
    return img


@pytest.mark.parametrize("w,h", [(64, 48), (123, 77), (200, 150)])
def test_resize_bit_exact(w, h):
    img = _img(w, h, w)
    sc = np.float32(2 ** 0.1)
    for ii in range(10):
        st = np.float32(1.0 / (float(sc) ** ii))
        a = O.resize(img, float(st)); b = O.ref_resize(img, float(st))
        assert a.shape == b.shape
        assert np.array_equal(a.view(np.int32), b.view(np.int32)), f"scale {st}"
    a = O.resize(img, 0.5); b = O.ref_resize(img, 0.5)
    assert np.array_equal(a.view(np.int32), b.view(np.int32))


@pytest.mark.parametrize("sbin", [4, 8])
@pytest.mark.parametrize("w,h", [(64, 48), (131, 99)])
def test_calc_feature_bit_exact(sbin, w, h):
    img = O.resize(_img(w, h, 7 + sbin), 0.83)
    a = O.calc_feature(img, sbin); b = O.ref_calc_feature(img, sbin)
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.int32), b.view(np.int32))


def test_max_scale(car_paths, person_paths):
    for paths in (car_paths, person_paths):
        m = O.Model(*paths)
        rs = [m.m.rsize[i] for i in range(2 * m.m.numcomponent)]
        for (w, h) in [(320, 240), (640, 480), (1280, 720), (1920, 1080), (100, 80)]:
            assert m.max_scale(w, h) == O.ref_max_scale(m.m.numcomponent, 8, 10, rs, w, h)


@pytest.mark.parametrize("seed", range(6))
def test_dt_bit_exact(seed):
    rng = np.random.default_rng(seed)
    d0, d1 = rng.integers(1, 60, size=2)
    vals = rng.normal(0, 0.3, size=(d1, d0)).astype(np.float32)
    if seed % 2:
        vals = np.round(vals * 4) / 4  # many exact ties
    a = rng.uniform(0.001 if seed < 4 else -0.05, 0.1, size=4).astype(np.float32)
    M, Ix, Iy = O.dt(vals, *a)
    rM, rIx, rIy = O.ref_dt(vals, *a)
    assert np.array_equal(M.view(np.int32), rM.view(np.int32))
    assert np.array_equal(Ix, rIx) and np.array_equal(Iy, rIy)


def test_add_part_and_boxes():
    rng = np.random.default_rng(3)
    score = rng.normal(size=(20, 9)).astype(np.float32)
    M = rng.normal(size=(45, 24)).astype(np.float32)
    for ax, ay in [(2, 2), (3, 5), (5, 1)]:
        s = score.copy()
        O.lib().orc_add_part(O._ptr(s), O._ptr(M), O._ptr(O._i32([9, 20])), O._ptr(O._i32([24, 45])), ax, ay)
        assert np.array_equal(s, O.ref_add_part(score, M, ax, ay))
    Ix = rng.integers(0, 45, size=(45, 24)).astype(np.int32)
    Iy = rng.integers(0, 24, size=(45, 24)).astype(np.int32)
    for scale in (np.float32(8.0), np.float32(8 / 0.5358867), np.float32(35.3)):
        for x, y in [(1, 1), (4, 7), (12, 3)]:
            a = np.zeros(4, np.float32)
            O.lib().orc_rootbox(x, y, float(scale), 0, 0, O._ptr(O._i32([6, 16])), O._ptr(a))
            assert np.array_equal(a, O.ref_rootbox(x, y, float(scale), [6, 16]))
            a = np.zeros(4, np.float32)
            O.lib().orc_partbox(x, y, 3, 2, float(scale), 0, 0, O._ptr(O._i32([6, 6])), O._ptr(Ix), O._ptr(Iy),
                                O._ptr(O._i32([24, 45])), O._ptr(a))
            assert np.array_equal(a, O.ref_partbox(x, y, 3, 2, float(scale), [6, 6], Ix, Iy))


def test_calc_a_score_and_gmpc():
    rng = np.random.default_rng(5)
    score = rng.normal(size=(30, 20)).astype(np.float32)
    for scale in (np.float32(8.0), np.float32(8 / 0.7578582), np.float32(8 / 0.1337)):
        ac = np.full((160, 120), -100, np.float32)
        a = ac.copy()
        O.lib().orc_calc_a_score(O._ptr(a), O._ptr(score), O._ptr(O._i32([20, 30])), O._ptr(O._i32([6, 16])),
                                 120, 160, 0, 0, float(scale))
        assert np.array_equal(a, O.ref_calc_a_score(ac, score, [6, 16], 120, 160, 8, float(scale)))
    g = O.ref_get_gmpc(score, 0.3)
    ys, xs = np.nonzero(score.T > np.float32(0.3))  # column-major scan: x outer, y inner
    order = np.lexsort((ys, xs))
    assert np.array_equal(g, np.stack([ys[order], xs[order]], 1))


@pytest.mark.parametrize("seed", range(5))
def test_quicksort_and_nms_with_ties(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 400))
    vals = np.round(rng.normal(size=n) * (2 if seed % 2 else 50)) / 4
    a, o = O.quicksort(vals); ra, ro = O.ref_quicksort(vals)
    assert np.array_equal(a, ra) and np.array_equal(o, ro)
    GL = 39
    boxes = np.zeros((n, GL), np.float32)
    xy = rng.uniform(0, 300, size=(n, 2)); wh = rng.uniform(10, 120, size=(n, 2))
    boxes[:, 0], boxes[:, 1] = xy[:, 1], xy[:, 0]
    boxes[:, 2], boxes[:, 3] = xy[:, 1] + wh[:, 1], xy[:, 0] + wh[:, 0]
    boxes[:, GL - 2] = vals
    boxes[:, GL - 1] = np.arange(n)  # unique rows
    keep, _, k = O.nms_keep(boxes, 0.5)
    rkeep, rk = O.ref_nms_keep(boxes, 8, 0.5)
    assert k == rk and np.array_equal(keep, rkeep)


def test_pyramid_matches_reference_functions(car_paths):
    """The oracle's pyramid orchestration (restated from featurepyramid.cpp.org)
    composed from the reference's own resize and calc_feature."""
    from geye_gb300 import synth
    m = O.Model(*car_paths)
    fr = synth.make_frame(160, 120, seed=3)
    P = O.Pyramid(m, fr)
    img0 = O.ipl_to_float(fr)
    sc = np.float32(2.0 ** (1.0 / 10))
    base = {}
    for ii in range(10):
        st = np.float32(1.0 / (float(sc) ** ii))
        base[ii] = O.ref_resize(img0, float(st))
    imgs = dict(base)
    for ii in range(10):
        cur = base[ii]
        for jj in range(ii + 10, P.LEN - 10, 10):
            cur = O.ref_resize(cur, 0.5)
            imgs[jj + 10] = cur
    for l in range(P.LEN):
        im = imgs[l] if l < 10 or l >= 20 else imgs[l - 10]
        f = O.ref_calc_feature(im, 4 if l < 10 else 8)
        assert np.array_equal(P.feat(l).view(np.int32), f.view(np.int32)), f"level {l}"


@pytest.mark.parametrize("n0,n1", [(1, 1), (5, 7), (23, 40)])
def test_flip_feat_bit_exact(n0, n1):
    f = np.random.default_rng(n0 * 100 + n1).normal(size=(31, n1, n0)).astype(np.float32)
    assert np.array_equal(O.flip_feat(f).view(np.int32), O.ref_flip_feat(f).view(np.int32))
