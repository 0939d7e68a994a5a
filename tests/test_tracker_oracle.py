"""CPU checks of the tracker restatement (oracle/tracker.py) itself."""
import numpy as np

from oracle import tracker as TR


def test_philox_normals_are_standard():
    z = TR.normals4(np.arange(200000, dtype=np.uint32), 0, 1, 3, *TR.keys(5))
    for a in z:
        assert abs(a.mean()) < 0.01 and abs(a.std() - 1.0) < 0.01


def test_philox_streams_differ_and_repeat():
    a = TR.philox4x32_10(np.arange(8, dtype=np.uint32), 0, 1, 0, *TR.keys(0))
    b = TR.philox4x32_10(np.arange(8, dtype=np.uint32), 0, 1, 0, *TR.keys(1))
    c = TR.philox4x32_10(np.arange(8, dtype=np.uint32), 0, 1, 0, *TR.keys(0))
    assert not np.array_equal(a[0], b[0]) and np.array_equal(a[0], c[0])


def test_tracker_follows_a_moving_box():
    tr = TR.StreamTracker(0)
    for k in range(12):
        tr.step(np.array([[100 + 3 * k, 50, 160 + 3 * k, 130]], float))
    b = tr.boxes()
    assert len(b) == 1 and abs(b[0][0] - 133) < 6 and abs(b[0][2] - 193) < 6
    for _ in range(TR.MAX_MISSED + 1):
        tr.step(np.zeros((0, 4)))
    assert len(tr.boxes()) == 0


def test_ascore_weights_the_particles():
    """A frame without an associated detection: particles on high A_SCORE pull
    the estimate (the reference adds A_SCORE to each particle's confidence)."""
    box = np.array([[100, 50, 160, 130]], float)
    plain, lit = TR.StreamTracker(0), TR.StreamTracker(0)
    for tr in (plain, lit):
        tr.step(box)
        tr.step(box)
    asc = np.zeros((1, 320, 240), np.float32)
    asc[0, 135:, :] = 1.0    # everything right of x = 135 scores 1
    plain.step(np.zeros((0, 4)))
    lit.step(np.zeros((0, 4)), asc)
    assert lit.boxes()[0][0] > plain.boxes()[0][0] + 1.0
    assert np.array_equal(TR.ascore_at(asc, np.array([-0.5, 134.9, 135.0, 320.0]), np.array([5.0, 5.0, 5.0, 5.0])),
                          [0.0, 0.0, 1.0, 0.0])
