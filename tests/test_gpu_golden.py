"""The CUDA stage entry points against the reference's own outputs recorded in
tests/golden/ref_vectors.npz (tests/golden/make_golden.py): resize,
calc_feature, flip_feat, dt and nms, bit-exact."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_vectors.npz")


@pytest.fixture(scope="module")
def V():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def ctx():
    import geye_gb300 as g
    c = g.Context(0)
    yield c
    c.close()


def _bits(a):
    a = np.asarray(a)
    return a.view(np.int32) if a.dtype == np.float32 else a


def test_resize(ctx, V):
    for k, s in enumerate(V["resize_scales"]):
        got = ctx.resize(V["resize_in"], float(s))
        assert got.shape == V[f"resize_out{k}"].shape
        assert np.array_equal(_bits(got), _bits(V[f"resize_out{k}"])), f"scale {s}"


def test_calc_feature(ctx, V):
    for sbin in (4, 8):
        got = ctx.calc_feature(V["feat_in"], sbin)
        assert np.array_equal(_bits(got), _bits(V[f"feat_out{sbin}"])), f"sbin {sbin}"


def test_flip_feat(ctx, V):
    assert np.array_equal(_bits(ctx.flip_feat(V["flip_in"])), _bits(V["flip_out"]))


def test_dt(ctx, V):
    for k in range(4):
        M, Ix, Iy = ctx.dt(V[f"dt_in{k}"], *[float(c) for c in V[f"dt_coef{k}"]])
        assert np.array_equal(_bits(M), _bits(V[f"dt_M{k}"])), f"case {k}"
        assert np.array_equal(Ix, V[f"dt_Ix{k}"]) and np.array_equal(Iy, V[f"dt_Iy{k}"]), f"case {k}"


def test_nms(ctx, V):
    for k in range(3):
        boxes = V[f"nms_in{k}"]
        want = boxes[V[f"nms_keep{k}"].astype(bool)]
        got = ctx.nms(boxes, 0.5, 8)
        assert got.shape == want.shape and np.array_equal(_bits(got), _bits(want)), f"case {k}"


def test_flip_feat_edges(ctx):
    """Empty maps give an empty result; a channel count other than 31 is rejected (the reference's ORD table has 31)."""
    import geye_gb300 as g
    out = ctx.flip_feat(np.zeros((31, 0, 5), np.float32))
    assert out.shape == (31, 0, 5)
    with pytest.raises(g.GeyeError):
        ctx.flip_feat(np.zeros((30, 4, 4), np.float32))
