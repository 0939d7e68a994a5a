"""The tensor-core convolution with FP8-e4m3 operands and per-filter scaling.

Features are stored times 256 and each filter times the power of two s_f that
brings its absolute maximum under 448 (e4m3's largest finite value); the
epilogue multiplies the FP32 accumulator by 1 / (256 s_f), which is exact.
e4m3 keeps 4 significant bits: a normal value rounds within a relative 2**-4,
a subnormal one within 2**-10 absolute (in scaled units).  So every map value
is within 0.13 * sum|a*b| + 2**-18 * sum|b| + 2**-10 / s_f * sum|a| of the
FP32 result.  Features that are multiples of 1/4 up to 1 and small integer
filters are exact in e4m3 after scaling, and their sums are exact in FP32,
so those maps must be bit-identical: that case pins the operand layouts.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx8():
    import geye_gb300 as g
    c = g.Context(0, conv=g.CONV_FP8)
    yield c
    c.close()


def _filter_scale(f):
    m = float(np.abs(f).max())
    return 1.0 if m == 0 else 2.0 ** np.floor(np.log2(448.0 / m))


def _maps_within_bound(got, feat, filters):
    for m, f in zip(got, filters):
        ref = O.fconv(feat, f)
        mag = O.fconv(np.abs(feat), np.abs(f))
        sum_b = O.fconv(np.ones_like(feat), np.abs(f))
        sum_a = O.fconv(np.abs(feat), np.ones_like(f))
        bound = 0.13 * mag + 2.0 ** -18 * sum_b + 2.0 ** -10 / _filter_scale(f) * sum_a + 1e-7
        err = np.abs(m.astype(np.float64) - ref.astype(np.float64))
        assert np.all(err <= bound), float((err / (mag + 1e-12)).max())


def test_fp8_exact_values_are_bit_identical(ctx8):
    rng = np.random.default_rng(5)
    feat = (rng.integers(0, 5, size=(31, 41, 37)) * 0.25).astype(np.float32)
    shapes = [(6, 6), (6, 6), (6, 16), (8, 13), (11, 5)]
    filters = [rng.integers(-2, 3, size=(31, b1, b0)).astype(np.float32) for b0, b1 in shapes]
    filters[1] *= 0.125   # another per-filter scale
    got = ctx8.fconvsMT(feat, filters)
    for m, f in zip(got, filters):
        assert np.array_equal(m, O.fconv(feat, f))


@pytest.mark.parametrize("nparts", [1, 16, 24])
def test_fp8_maps_within_rounding_bound(ctx8, nparts):
    rng = np.random.default_rng(100 + nparts)
    feat = (rng.random((31, 78, 58)) * 0.4).astype(np.float32)
    filters = [rng.normal(0, 0.01, size=(31, 6, 6)).astype(np.float32) for _ in range(nparts)]
    filters += [rng.normal(0, 0.01, size=(31, 16, 6)).astype(np.float32)]
    _maps_within_bound(ctx8.fconvsMT(feat, filters), feat, filters)


def test_fp8_filter_columns_in_phases(ctx8):
    rng = np.random.default_rng(13)
    feat = (rng.integers(0, 5, size=(31, 60, 640)) * 0.25).astype(np.float32)
    filters = [rng.integers(-2, 3, size=(31, 16, 6)).astype(np.float32) for _ in range(3)]
    got = ctx8.fconvsMT(feat, filters)
    for m, f in zip(got, filters):
        assert np.array_equal(m, O.fconv(feat, f))
