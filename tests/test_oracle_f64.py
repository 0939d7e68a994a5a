"""The double-precision score restatement against the FP32 oracle.

The FP64 score (convolutions, distance transforms and part sum in double from
the same FP32 features) measures the error of the reduced-precision paths; it
must agree with the FP32 oracle's score maps to within FP32 rounding of the
sums (2**-20 of the magnitude bound), level by level and component by component.
"""
import numpy as np

from geye_gb300 import synth
from oracle import oracle as O


def test_f64_scores_match_fp32_oracle(tmp_path):
    paths = synth.write_model_csv(synth.CAR_SPEC, str(tmp_path))
    m = O.Model(*paths)
    frame = synth.make_frame(224, 168, seed=4)
    P = O.Pyramid(m, frame)
    S = O.Scores(m, P)
    checked = 0
    for level in range(S.interval, S.LEN):
        if S.skipped[level]:
            continue
        for c in range(S.NoC):
            r = S.score_f64(level, c)
            assert r is not None
            s64, mag = r
            s32 = S.score(level, c).astype(np.float64)
            assert s64.shape == s32.shape
            assert mag > 0
            assert np.abs(s64 - s32).max() <= 2.0 ** -20 * mag + 1e-6
            checked += 1
    assert checked >= 4
