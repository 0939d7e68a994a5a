"""The argument behind the pipeline NMS's score order (geye_gb300/csrc/nms_radix.cu),
checked on the CPU with the oracle: resolving the boxes in score order (equal
scores by input index) gives nms.cpp's kept set -- the order of the reference's
quicksort (nms.cpp:70-84) -- unless

  (a) a pick suppresses an alive box of its own run of equal scores, or
  (b) the last pick shares its score with another pick,

and those are exactly the cases the pipeline hands to the quicksort-order pass.
The restatement below walks the boxes sequentially (the GPU decides the same
boxes in batches); its suppression test is nms.cpp's with its float roundings."""
import numpy as np
import pytest

from geye_gb300 import synth
from oracle import oracle as O


def _areas(b):
    x1, y1, x2, y2 = b[:, 1], b[:, 0], b[:, 3], b[:, 2]
    return (((x2 - x1).astype(np.float64) + 1.0) * ((y2 - y1).astype(np.float64) + 1.0)).astype(np.float32)


def _suppressed(b, ar, i, overlap):
    y1, x1, y2, x2 = (b[:, k] for k in range(4))
    yy1, xx1 = np.maximum(y1[i], y1), np.maximum(x1[i], x1)
    yy2, xx2 = np.minimum(y2[i], y2), np.minimum(x2[i], x2)
    w = (xx2 - xx1 + np.float32(1)).astype(np.float32)
    h = (yy2 - yy1 + np.float32(1)).astype(np.float32)
    cont = ((y1[i] < y1) & (x1[i] < x1) & (y2[i] > y2) & (x2[i] > x2)) | \
           ((y1[i] > y1) & (x1[i] > x1) & (y2[i] < y2) & (x2[i] < x2))
    ratio = (w * h / np.minimum(ar[i], ar)).astype(np.float32)
    return np.where((w > 0) & (h > 0), ratio > np.float32(overlap), cont)


def key_order_nms(boxes, overlap):
    """(keep mask in input order, needs the quicksort's order)"""
    b = np.ascontiguousarray(boxes, np.float32)
    D = len(b)
    sc = b[:, -2]
    order = np.lexsort((np.arange(D), -sc.astype(np.float64)))
    ar = _areas(b)
    alive = np.ones(D, bool)
    picks, hit_any, need = [], [], bool(np.isnan(sc).any())
    for i in order:
        if not alive[i]:
            continue
        alive[i] = False
        s = _suppressed(b, ar, i, overlap)
        hit = s & alive
        if np.any(hit & (sc == sc[i])):
            need = True   # (a)
        hit_any.append(bool(hit.any()))
        alive &= ~s
        picks.append(i)
    if len(picks) >= 2 and sc[picks[-1]] == sc[picks[-2]]:
        need = True       # (b)
    keep = np.zeros(D, bool)
    k = len(picks) - (1 if picks and not hit_any[-1] else 0)   # the box alone at its turn is never emitted
    keep[picks[:k]] = True
    return keep, need


@pytest.mark.parametrize("w,h,seed", [(320, 240, 1), (640, 480, 0), (640, 480, 1)])
def test_score_order_gives_the_quicksort_kept_set(car_paths, person_paths, w, h, seed):
    fr = synth.make_frame(w, h, seed=seed)
    for paths in (car_paths, person_paths):
        boxes = O.car_detection(O.Model(*paths), fr, -0.5, 0.5)["boxes"]
        keep, need = key_order_nms(boxes, 0.5)
        ref, _, _ = O.nms_keep(boxes, 0.5)
        if not need:   # else the pipeline resolves this model again in the quicksort's order
            assert np.array_equal(keep, ref)


def _run_boxes(scores, boxes):
    """records [y1, x1, y2, x2, comp, score, scale] (GL = 7)"""
    out = np.zeros((len(boxes), 7), np.float32)
    out[:, :4] = boxes
    out[:, 5] = scores
    out[:, 6] = 1.0
    return out


def test_a_run_whose_boxes_suppress_each_other_needs_the_quicksort_order():
    """Five boxes of one score sliding by 8 px, two lower isolated boxes after them:
    which of the run's boxes is picked first is the quicksort's call, and the
    score order's choice differs from it here."""
    run = [[104, 808 + 8 * k, 151, 935 + 8 * k] for k in range(5)]
    boxes = _run_boxes([0.3] * 5 + [0.1, 0.05], run + [[10, 10, 60, 60], [300, 300, 350, 350]])
    rng = np.random.default_rng(3)
    differs = 0
    for _ in range(20):   # the run's members in other input positions
        perm = rng.permutation(len(boxes))
        b = boxes[perm]
        keep, need = key_order_nms(b, 0.5)
        ref, _, _ = O.nms_keep(b, 0.5)
        assert need
        differs += not np.array_equal(keep, ref)
    assert differs > 0   # the flag is needed: score order alone would be wrong for some inputs


def test_last_picks_of_equal_score_need_the_quicksort_order():
    """Two isolated boxes of the lowest score: the last pick's run holds another
    pick, and which of them the reference drops as alone at its turn is the
    quicksort's call."""
    boxes = _run_boxes([0.9, 0.2, 0.2], [[0, 0, 50, 50], [100, 100, 150, 150], [300, 300, 350, 350]])
    keep, need = key_order_nms(boxes, 0.5)
    assert need and keep.sum() == 2


def test_distinct_scores_never_need_it():
    rng = np.random.default_rng(11)
    xy = rng.uniform(0, 600, size=(400, 2)).astype(np.float32)
    wh = rng.uniform(20, 120, size=(400, 2)).astype(np.float32)
    boxes = _run_boxes(rng.permutation(400).astype(np.float32) / 400.0,
                       np.concatenate([xy[:, 1:2], xy[:, 0:1], xy[:, 1:2] + wh[:, 1:2], xy[:, 0:1] + wh[:, 0:1]], 1))
    keep, need = key_order_nms(boxes, 0.5)
    ref, _, _ = O.nms_keep(boxes, 0.5)
    assert not need and np.array_equal(keep, ref)
