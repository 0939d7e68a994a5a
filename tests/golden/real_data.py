"""The reference's own test data as fixtures: its 21 test frames
(CAR_TRACKING/Test_Images/org_image/{0..20}.png, decoded by geye_gb300.png)
and its trained car and person models (CAR_TRACKING/{car,person}_*.csv, as
the reference's loader parses them), with the oracle's detections on every
frame for each model.  tests/golden/make_real_golden.py writes the three .npz
files from the reference checkout; this module reads them back on machines
that have only this repository.

Files:
  real_frames.npz    frames_dx: (21, 480, 640, 3) uint8, each row stored as
                     differences along x modulo 256 (undone by a running sum)
  real_models.npz    <name>_dump: every field the reference's loader parses,
                     flattened as oracle/ref/ref_glue.cpp ref_load_model_dump
                     writes them
  real_expected.npz  per model and frame: the oracle's kept records and
                     RESULT fields, the box count before NMS, the SHA-256
                     of the A_SCORE map's float bits and of every (level,
                     component) score map's (score_maps lists the pairs);
                     gnr_<name>_boxes and gnr_<name>_<ratio>_<field>: the
                     reference's own get_new_rects on kept records (and on
                     those records moved past the image borders)
"""
from __future__ import annotations

import hashlib
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FRAMES = os.path.join(HERE, "real_frames.npz")
MODELS = os.path.join(HERE, "real_models.npz")
EXPECTED = os.path.join(HERE, "real_expected.npz")

MODEL_NAMES = ("car", "person")
N_FRAMES = 21
# the reference's run parameters (CAR_TRACKING/main.cpp:86-88)
THRESH = -0.5
OVERLAP = 0.4
RATIO = 1.0
# model ratios at which the reference's get_new_rects is recorded (or_point = point / ratio)
GNR_RATIOS = (1.0, 0.75)


def encode_frames(frames: np.ndarray) -> np.ndarray:
    d = frames.astype(np.int16)
    d[:, :, 1:, :] -= frames[:, :, :-1, :].astype(np.int16)
    return (d & 0xFF).astype(np.uint8)


def decode_frames(dx: np.ndarray) -> np.ndarray:
    return np.cumsum(dx, axis=2, dtype=np.uint8)


def load_frames() -> np.ndarray:
    """(21, 480, 640, 3) uint8 B,G,R frames, as the reference's IplImage holds them."""
    return np.ascontiguousarray(decode_frames(np.load(FRAMES)["frames_dx"]))


def float_digest(a_score: np.ndarray) -> bytes:
    return hashlib.sha256(np.ascontiguousarray(a_score, np.float32).view(np.uint32).tobytes()).digest()


def parse_dump(dump: np.ndarray) -> dict:
    """The flat loader dump -> the loader's fields (names of CAR_TRACKING/MODEL_info.h:75-142)."""
    v = [float(x) for x in dump]
    pos = 0

    def take(n=1):
        nonlocal pos
        out = v[pos:pos + n]
        pos += n
        return out if n != 1 else out[0]

    def ti(n=1):
        r = take(n)
        return [int(x) for x in r] if n != 1 else int(r)

    f = dict(numcomponent=ti(), sbin=ti(), interval=ti(), max_Y=ti(), max_X=ti(), padx=ti(), pady=ti())
    f["comps"] = []
    for _ in range(f["numcomponent"]):
        c = dict(ridx=ti(), oidx=ti(), offw=np.float32(take()), rsize=ti(2), numpart=ti())
        c["parts"] = [dict(pidx=ti(), didx=ti(), psize=ti(2)) for _ in range(c["numpart"])]
        f["comps"].append(c)
    defl = ti()
    f["def"] = np.array(take(4 * defl), np.float32).reshape(defl, 4)
    f["anchor"] = np.array(ti(2 * defl), np.int32).reshape(defl, 2)
    for c in f["comps"]:
        gl = 1 + 2 * (1 + c["numpart"])
        for k in ("x1", "y1", "x2", "y2"):
            c[k] = np.array(take(gl), np.float32)
    f["roots"] = []
    for _ in range(ti()):
        size = ti(3)
        sym = ti()
        f["roots"].append(dict(size=size, sym=sym, w=np.array(take(size[0] * size[1] * size[2]), np.float32)))
    f["parts"] = []
    for _ in range(ti()):
        size = ti(3)
        partner, psym = ti(), ti()
        f["parts"].append(dict(size=size, partner=partner, sym=psym,
                               w=np.array(take(size[0] * size[1] * size[2]), np.float32)))
    assert pos == len(v), (pos, len(v))
    return f


def _line(vals) -> str:
    # %.9g reproduces every float32 exactly through the loader's fscanf("%f,")
    return "".join(f"{float(np.float32(x)):.9g},\n" for x in vals)


def write_model_csv(dump: np.ndarray, out_dir: str, name: str) -> tuple[str, str, str]:
    """Writes the model the dump describes as a CSV triple in the reference's
    format (CAR_TRACKING/load_model.cpp:57-530) and returns the three paths."""
    f = parse_dump(dump)
    comp = [f["numcomponent"], f["sbin"], f["interval"], f["max_Y"], f["max_X"]]
    for c in f["comps"]:
        comp += [c["ridx"] + 1, c["oidx"] + 1, c["offw"], *c["rsize"], c["numpart"]]
        for p in c["parts"]:
            comp += [p["pidx"] + 1, p["didx"] + 1, *p["psize"]]
    comp += [len(f["def"])]
    for d, a in zip(f["def"], f["anchor"]):
        comp += [*d, *a]
    for c in f["comps"]:
        comp += [*c["x1"], *c["y1"], *c["x2"], *c["y2"]]
    root = [len(f["roots"])]
    for r in f["roots"]:
        root += [*r["size"], *r["w"]]
    part = [len(f["parts"])]
    for p in f["parts"]:
        part += [*p["size"], *p["w"], p["partner"]]
    os.makedirs(out_dir, exist_ok=True)
    paths = tuple(os.path.join(out_dir, f"{name}_{kind}.csv") for kind in ("comp", "root", "part"))
    for p, vals in zip(paths, (comp, root, part)):
        with open(p, "w") as fh:
            fh.write(_line(vals))
    return paths


def model_dump(name: str) -> np.ndarray:
    return np.load(MODELS)[f"{name}_dump"]


def get_new_rects_vectors(name: str) -> tuple:
    """(boxes, {ratio: RESULT fields}) recorded from the reference's get_new_rects."""
    E = np.load(EXPECTED)
    out = {ratio: {k: E[f"gnr_{name}_{ratio}_{k}"] for k in ("point", "or_point", "type", "scale", "score")}
           for ratio in GNR_RATIOS}
    return E[f"gnr_{name}_boxes"], out


def expected(name: str, frame: int) -> dict:
    E = np.load(EXPECTED)
    k = f"{name}_{frame}_"
    return {key[len(k):]: E[key] for key in E.files if key.startswith(k)}
