"""Writes the real-data fixtures of tests/golden/real_data.py from a checkout
of the reference (GEYE_REF_DIR, else ../reference/CAR_TRACKING beside this
repository):

  - the 21 test frames CAR_TRACKING/Test_Images/org_image/{0..20}.png,
    decoded by geye_gb300.png (zlib inflate and the five PNG row filters);
  - the trained car and person models, parsed by the reference's own loader
    (load_model.cpp, compiled into oracle/_ref); the CSV triple rewritten from
    that parse is checked to parse back to the same fields;
  - the oracle's detections (thresh -0.5, overlap 0.4, ratio 1: the
    reference's run parameters, CAR_TRACKING/main.cpp:86-88) for every frame
    and model, with the digests of the A_SCORE map and of every (level,
    component) score map;
  - the reference's own get_new_rects (tracking.cpp, compiled into
    oracle/_ref) on every kept record and on those records moved past the
    image borders, at two model ratios.

Run from the repository root:  python tests/golden/make_real_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from geye_gb300 import png  # noqa: E402
from oracle import oracle as O  # noqa: E402
import real_data as RD  # noqa: E402


def main() -> None:
    if O.ref_lib() is None:
        raise SystemExit("the reference sources are needed (GEYE_REF_DIR)")
    src = O.REF_SRC_DIR
    frames = np.stack([png.load_bgr(os.path.join(src, "Test_Images", "org_image", f"{i}.png"))
                       for i in range(RD.N_FRAMES)])
    np.savez_compressed(RD.FRAMES, frames_dx=RD.encode_frames(frames))
    assert np.array_equal(RD.load_frames(), frames)

    dumps = {}
    with tempfile.TemporaryDirectory() as d:
        for name in RD.MODEL_NAMES:
            paths = [os.path.join(src, f"{name}_{k}.csv") for k in ("comp", "root", "part")]
            dumps[name] = O.ref_load_model(*paths)
            again = O.ref_load_model(*RD.write_model_csv(dumps[name], d, name))
            assert np.array_equal(again.view(np.uint32), dumps[name].view(np.uint32)), name
    np.savez_compressed(RD.MODELS, **{f"{n}_dump": v for n, v in dumps.items()})

    E = {}
    with tempfile.TemporaryDirectory() as d:
        for name in RD.MODEL_NAMES:
            m = O.Model(*[os.path.join(src, f"{name}_{k}.csv") for k in ("comp", "root", "part")], RD.RATIO)
            for i in range(RD.N_FRAMES):
                a = np.full((640, 480), -100, np.float32)
                r = O.car_detection(m, frames[i], RD.THRESH, RD.OVERLAP, a_score=a)
                k = f"{name}_{i}_"
                for key in ("kept", "point", "or_point", "type", "scale", "score"):
                    E[k + key] = r[key]
                E[k + "D"] = np.int32(r["D"])
                E[k + "probe_oob"] = np.int32(r["probe_oob"])
                E[k + "a_score_sha256"] = np.frombuffer(RD.float_digest(a), np.uint8)
                S = O.Scores(m, O.Pyramid(m, frames[i]))
                maps = [(lv, c) for lv in range(S.interval, S.LEN) if not S.skipped[lv] for c in range(S.NoC)]
                E[k + "score_maps"] = np.array(maps, np.int32)
                E[k + "score_sha256"] = np.stack([np.frombuffer(RD.float_digest(S.score(lv, c)), np.uint8)
                                                  for lv, c in maps])
                print(name, i, "D", r["D"], "kept", r["K"], "oob", r["probe_oob"])
    # get_new_rects (tracking.cpp:90-166) by the reference's own function: every
    # kept record of every frame, and those records moved past each image border
    # (the clamps) and to negative coordinates, at ratios 1 and 0.75 (or_point)
    for name in RD.MODEL_NAMES:
        paths = [os.path.join(src, f"{name}_{k}.csv") for k in ("comp", "root", "part")]
        kept = np.concatenate([E[f"{name}_{i}_kept"] for i in range(RD.N_FRAMES)])
        moved = []
        for dx, dy in ((-300.0, 0.0), (400.0, 0.0), (0.0, -250.0), (0.0, 300.0), (-500.0, -400.0)):
            k2 = kept.copy()
            k2[:, 0:kept.shape[1] - 3:4] += dy   # y1 of the root and every part box
            k2[:, 2:kept.shape[1] - 3:4] += dy   # y2
            k2[:, 1:kept.shape[1] - 3:4] += dx   # x1
            k2[:, 3:kept.shape[1] - 3:4] += dx   # x2
            moved.append(k2)
        boxes = np.concatenate([kept] + moved).astype(np.float32)
        E[f"gnr_{name}_boxes"] = boxes
        for ratio in RD.GNR_RATIOS:
            r = O.ref_get_new_rects(*paths, ratio, boxes, 640, 480)
            for key in ("point", "or_point", "type", "scale", "score"):
                E[f"gnr_{name}_{ratio}_{key}"] = r[key]
    np.savez_compressed(RD.EXPECTED, **E)
    for p in (RD.FRAMES, RD.MODELS, RD.EXPECTED):
        print(p, os.path.getsize(p), "bytes")


if __name__ == "__main__":
    main()
