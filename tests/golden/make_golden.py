"""Writes tests/golden/ref_vectors.npz: seeded inputs and the outputs of the
reference's own CPU functions (CAR_TRACKING sources compiled into oracle/_ref
by oracle/ref/Makefile) for them.

The reference ships no test vectors; these fixtures carry its results to
machines without its sources, where tests/test_golden.py checks
the oracle and tests/test_gpu_golden.py checks the CUDA stage entry points
against them.  Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_vectors.npz")


def _img(w, h, seed):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, size=(3, w, h)).astype(np.float32)
    img[:, : w // 3, : h // 3] = 77.0   # a flat patch: exact ties and zero gradients
    return img


def main() -> None:
    if O.ref_lib() is None:
        raise SystemExit("the reference sources are needed to build oracle/_ref")
    V: dict[str, np.ndarray] = {}

    # resize (resize.cc:135-160): the base-octave scales 1/sc^i and the octave step 0.5
    img = _img(64, 48, 1)
    V["resize_in"] = img
    sc = np.float32(2 ** 0.1)
    scales = [np.float32(1.0 / (float(sc) ** i)) for i in (1, 3, 7)] + [np.float32(0.5)]
    V["resize_scales"] = np.array(scales, np.float32)
    for k, s in enumerate(scales):
        V[f"resize_out{k}"] = O.ref_resize(img, float(s))

    # calc_feature (featurepyramid.cpp:263-501), sbin 4 and 8
    fimg = O.ref_resize(_img(72, 56, 2), 0.83)
    V["feat_in"] = fimg
    for sbin in (4, 8):
        V[f"feat_out{sbin}"] = O.ref_calc_feature(fimg, sbin)

    # flip_feat (get_boxes.cpp:121-178)
    ff = np.random.default_rng(3).normal(size=(31, 7, 5)).astype(np.float32)
    V["flip_in"] = ff
    V["flip_out"] = O.ref_flip_feat(ff)

    # dt (dt.cpp:61-136): smooth values, quarter-step ties, and a negative coefficient
    for k in range(4):
        rng = np.random.default_rng(10 + k)
        d0, d1 = (int(v) for v in rng.integers(5, 40, size=2))
        vals = rng.normal(0, 0.3, size=(d1, d0)).astype(np.float32)
        if k % 2:
            vals = (np.round(vals * 4) / 4).astype(np.float32)
        coef = rng.uniform(0.001 if k < 3 else -0.05, 0.1, size=4).astype(np.float32)
        M, Ix, Iy = O.ref_dt(vals, *coef)
        V[f"dt_in{k}"], V[f"dt_coef{k}"] = vals, coef
        V[f"dt_M{k}"], V[f"dt_Ix{k}"], V[f"dt_Iy{k}"] = M, Ix, Iy

    # quickSort (nms.cpp:70-84) with many equal keys, and nms (nms.cpp:94-217)
    for k in range(3):
        rng = np.random.default_rng(20 + k)
        n = (1, 57, 300)[k]
        vals = (np.round(rng.normal(size=n) * (2 if k % 2 else 40)) / 4).astype(np.float32)
        a, order = O.ref_quicksort(vals)
        V[f"qs_in{k}"], V[f"qs_val{k}"], V[f"qs_ord{k}"] = vals, a, order
        GL = 39
        boxes = np.zeros((n, GL), np.float32)
        xy = rng.uniform(0, 300, size=(n, 2))
        wh = rng.uniform(10, 120, size=(n, 2))
        boxes[:, 0], boxes[:, 1] = xy[:, 1], xy[:, 0]
        boxes[:, 2], boxes[:, 3] = xy[:, 1] + wh[:, 1], xy[:, 0] + wh[:, 0]
        boxes[:, GL - 2] = vals
        boxes[:, GL - 1] = np.arange(n)
        keep, kept = O.ref_nms_keep(boxes, 8, 0.5)
        V[f"nms_in{k}"], V[f"nms_keep{k}"] = boxes, keep.astype(np.int8)

    # add_part_calculation (dt.cpp:38-55), rootbox / partbox (get_boxes.cpp:227-258)
    rng = np.random.default_rng(30)
    score = rng.normal(size=(20, 9)).astype(np.float32)
    M = rng.normal(size=(45, 24)).astype(np.float32)
    V["ap_score"], V["ap_M"] = score, M
    for k, (ax, ay) in enumerate([(2, 2), (3, 5), (5, 1)]):
        V[f"ap_out{k}"] = O.ref_add_part(score, M, ax, ay)
    V["ap_anchor"] = np.array([(2, 2), (3, 5), (5, 1)], np.int32)
    Ix = rng.integers(0, 45, size=(45, 24)).astype(np.int32)
    Iy = rng.integers(0, 24, size=(45, 24)).astype(np.int32)
    V["pb_Ix"], V["pb_Iy"] = Ix, Iy
    bscales = np.array([8.0, 8 / 0.5358867, 35.3], np.float32)
    pts = np.array([(1, 1), (4, 7), (12, 3)], np.int32)
    V["box_scales"], V["box_pts"] = bscales, pts
    V["rootbox_out"] = np.array([[O.ref_rootbox(int(x), int(y), float(s), [6, 16]) for x, y in pts] for s in bscales])
    V["partbox_out"] = np.array([[O.ref_partbox(int(x), int(y), 3, 2, float(s), [6, 6], Ix, Iy) for x, y in pts]
                                 for s in bscales])

    # calc_a_score (get_boxes.cpp:265-300) and get_gmpc (get_boxes.cpp:185-223)
    rng = np.random.default_rng(40)
    sc_map = rng.normal(size=(30, 20)).astype(np.float32)
    V["as_score"] = sc_map
    as_scales = np.array([8.0, 8 / 0.7578582, 8 / 0.1337], np.float32)
    V["as_scales"] = as_scales
    for k, s in enumerate(as_scales):
        V[f"as_out{k}"] = O.ref_calc_a_score(np.full((160, 120), -100, np.float32), sc_map, [6, 16], 120, 160, 8,
                                             float(s))
    V["gmpc_out"] = O.ref_get_gmpc(sc_map, 0.3)

    # ini_scales' max_scale (featurepyramid.cpp:174-239) for the benchmark models' root sizes
    sizes = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (100, 80)]
    car_rs, person_rs = [6, 16, 8, 13], [11, 5, 10, 6, 9, 7]
    V["ms_sizes"] = np.array(sizes, np.int32)
    V["ms_car"] = np.array([O.ref_max_scale(2, 8, 10, car_rs, w, h) for w, h in sizes], np.int32)
    V["ms_person"] = np.array([O.ref_max_scale(3, 8, 10, person_rs, w, h) for w, h in sizes], np.int32)

    np.savez_compressed(OUT, **V)
    print(OUT, os.path.getsize(OUT), "bytes,", len(V), "arrays")


if __name__ == "__main__":
    main()
