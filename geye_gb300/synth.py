"""Seeded synthetic inputs for the DPM detection path.

Frames: a smooth value-noise texture (several octaves, smoothstep-interpolated
random lattices) with 20 filled rectangles of random colour on top, returned
as interleaved 8-bit BGR rows, the pixel layout of the reference's IplImage
input (CAR_TRACKING/featurepyramid.cpp.org:461-500 reads B, G, R at
widthStep*y + 3x).

Models: random-init DPM models written in the reference's three-file CSV
format (component / root / part files, parsed by
CAR_TRACKING/load_model.cpp:57-530), so the library and the oracle both load
them the way the reference loads its trained car and person models.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

__all__ = ["make_frame", "ModelSpec", "CAR_SPEC", "PERSON_SPEC", "CAR_TRAINED_LIKE", "PERSON_TRAINED_LIKE",
           "write_model_csv", "model_paths"]


def _value_noise(rng: np.random.Generator, h: int, w: int, cell: int) -> np.ndarray:
    gh, gw = h // cell + 2, w // cell + 2
    lat = rng.random((gh, gw))
    ys = np.arange(h) / cell
    xs = np.arange(w) / cell
    y0 = np.floor(ys).astype(np.int64)
    x0 = np.floor(xs).astype(np.int64)
    fy = ys - y0
    fx = xs - x0
    sy = fy * fy * (3 - 2 * fy)
    sx = fx * fx * (3 - 2 * fx)
    a = lat[y0][:, x0]
    b = lat[y0][:, x0 + 1]
    c = lat[y0 + 1][:, x0]
    d = lat[y0 + 1][:, x0 + 1]
    top = a + (b - a) * sx[None, :]
    bot = c + (d - c) * sx[None, :]
    return top + (bot - top) * sy[:, None]


def make_frame(width: int, height: int, seed: int = 0, n_rects: int = 20) -> np.ndarray:
    """Returns a (height, width, 3) uint8 BGR frame, C-contiguous (widthStep = 3*width)."""
    rng = np.random.default_rng(seed)
    img = np.zeros((height, width, 3), dtype=np.float64)
    for ch in range(3):
        acc = np.zeros((height, width))
        amp = 1.0
        tot = 0.0
        for cell in (96, 48, 24, 12):
            acc += amp * _value_noise(rng, height, width, cell)
            tot += amp
            amp *= 0.5
        img[:, :, ch] = acc / tot
    img = 40.0 + 175.0 * img
    for _ in range(n_rects):
        rw = int(rng.integers(max(4, width // 24), max(5, width // 3)))
        rh = int(rng.integers(max(4, height // 24), max(5, height // 3)))
        x0 = int(rng.integers(0, max(1, width - rw)))
        y0 = int(rng.integers(0, max(1, height - rh)))
        col = rng.integers(0, 256, size=3)
        img[y0:y0 + rh, x0:x0 + rw, :] = col[None, None, :]
    return np.ascontiguousarray(np.clip(np.rint(img), 0, 255).astype(np.uint8))


@dataclass
class ModelSpec:
    """Shape of a random-init DPM model.  Sizes are (rows/y, cols/x) in cells.

    With `parts` set (per component, a list of part sizes), the model follows the
    shapes and value statistics of a trained model: per-component part sizes,
    filter weights ~ N(0, root_std / part_std), component offsets `offsets`, and
    deformation weights drawn uniformly in `def_ranges` ((lo, hi) for ax, bx, ay, by).
    Without it: `parts_per_component` parts of `part_size`, weights ~ N(0, 0.01),
    offsets ~ N(0, 0.1), deformation weights ~ U(0.01, 0.1)."""
    name: str
    roots: list
    parts_per_component: int = 8
    part_size: tuple = (6, 6)
    sbin: int = 8
    interval: int = 10
    seed: int = 1
    extra: dict = field(default_factory=dict)
    parts: list | None = None
    root_std: float = 0.01
    part_std: float = 0.01
    offsets: list | None = None
    def_ranges: tuple | None = None


CAR_SPEC = ModelSpec("car", roots=[(6, 16), (8, 13)], seed=1)
PERSON_SPEC = ModelSpec("person", roots=[(11, 5), (10, 6), (9, 7)], seed=2)

# Shapes and value statistics of the reference's trained car and person models
# (CAR_TRACKING/car_*.csv, person_*.csv): root and part sizes per component,
# weight standard deviations, component offsets and deformation-weight ranges;
# the weights themselves are random.
CAR_TRAINED_LIKE = ModelSpec(
    "car_tl", roots=[(6, 13), (6, 7)], seed=11,
    parts=[[(9, 6), (9, 6), (6, 10), (10, 6), (10, 6), (9, 6)], [(7, 4), (7, 4), (5, 6), (5, 6), (5, 6), (7, 4)]],
    root_std=0.024, part_std=0.025, offsets=[-4.06, -3.84],
    def_ranges=((0.010, 0.034), (-0.011, 0.011), (0.015, 0.067), (-0.044, 0.037)))
PERSON_TRAINED_LIKE = ModelSpec(
    "person_tl", roots=[(9, 6), (11, 4)], seed=12,
    parts=[[(6, 6), (6, 6), (6, 6), (5, 8), (8, 5), (8, 5)], [(5, 6), (5, 6), (8, 4), (8, 4), (5, 6), (5, 6)]],
    root_std=0.038, part_std=0.037, offsets=[-3.87, -7.77],
    def_ranges=((0.010, 0.177), (-0.022, 0.022), (0.034, 0.156), (-0.069, 0.021)))


def _fmt(vals) -> str:
    return "".join(f"{float(v):14.6f},\n" for v in np.asarray(vals, dtype=np.float64).ravel())


def write_model_csv(spec: ModelSpec, out_dir: str) -> tuple[str, str, str]:
    """Writes <name>_comp.csv, <name>_root.csv, <name>_part.csv and returns their paths.

    Weights ~ N(0, 0.01); deformation weights (all four) ~ U(0.01, 0.1); the
    component offset ~ N(0, 0.1); anchors are drawn in [1, 2*root - part - 1]
    per axis so every part placement stays inside its part-score map.
    """
    os.makedirs(out_dir, exist_ok=True)
    if spec.parts is not None:
        return _write_trained_like(spec, out_dir)
    rng = np.random.default_rng(spec.seed)
    nc = len(spec.roots)
    npart = spec.parts_per_component
    ph, pw = spec.part_size
    max_y = max(r[0] for r in spec.roots)
    max_x = max(r[1] for r in spec.roots)
    comp = [nc, spec.sbin, spec.interval, max_y, max_x]
    defs = []
    for c, (rh, rw) in enumerate(spec.roots):
        comp += [c + 1, c + 1, rng.normal(0.0, 0.1), rh, rw, npart]
        for k in range(npart):
            idx = c * npart + k + 1
            comp += [idx, idx, ph, pw]
            dvals = rng.uniform(0.01, 0.1, size=4)
            axmax = max(1, 2 * rw - pw - 1)
            aymax = max(1, 2 * rh - ph - 1)
            anc = [int(rng.integers(1, axmax + 1)), int(rng.integers(1, aymax + 1))]
            defs.append((dvals, anc))
    comp += [len(defs)]
    for dvals, anc in defs:
        comp += list(dvals) + anc
    gl = 1 + 2 * (1 + npart)
    for c in range(nc):
        x1 = np.zeros(gl); x1[1] = 1.0
        y1 = np.zeros(gl); y1[2] = 1.0
        x2 = np.zeros(gl); x2[0] = 1.0; x2[1] = 1.0
        y2 = np.zeros(gl); y2[0] = 0.375; y2[2] = 1.0
        comp += list(x1) + list(y1) + list(x2) + list(y2)
    root = [nc]
    for (rh, rw) in spec.roots:
        root += [rh, rw, 31] + list(rng.normal(0.0, 0.01, size=rh * rw * 31))
    part = [nc * npart]
    for c in range(nc):
        for k in range(npart):
            part += [ph, pw, 31] + list(rng.normal(0.0, 0.01, size=ph * pw * 31)) + [0]
    paths = tuple(os.path.join(out_dir, f"{spec.name}_{kind}.csv") for kind in ("comp", "root", "part"))
    for p, vals in zip(paths, (comp, root, part)):
        with open(p, "w") as f:
            f.write(_fmt(vals))
    return paths


def _write_trained_like(spec: ModelSpec, out_dir: str) -> tuple[str, str, str]:
    rng = np.random.default_rng(spec.seed)
    nc = len(spec.roots)
    max_y = max(r[0] for r in spec.roots)
    max_x = max(r[1] for r in spec.roots)
    comp = [nc, spec.sbin, spec.interval, max_y, max_x]
    defs, psizes = [], []
    for c, (rh, rw) in enumerate(spec.roots):
        plist = spec.parts[c]
        comp += [c + 1, c + 1, spec.offsets[c], rh, rw, len(plist)]
        for (ph, pw) in plist:
            idx = len(psizes) + 1
            comp += [idx, idx, ph, pw]
            dvals = [rng.uniform(lo, hi) for lo, hi in spec.def_ranges]
            axmax = max(1, 2 * rw - pw - 1)
            aymax = max(1, 2 * rh - ph - 1)
            anc = [int(rng.integers(1, axmax + 1)), int(rng.integers(1, aymax + 1))]
            defs.append((dvals, anc))
            psizes.append((ph, pw))
    comp += [len(defs)]
    for dvals, anc in defs:
        comp += list(dvals) + anc
    npart = len(spec.parts[0])
    gl = 1 + 2 * (1 + npart)
    for c in range(nc):
        x1 = np.zeros(gl); x1[1] = 1.0
        y1 = np.zeros(gl); y1[2] = 1.0
        x2 = np.zeros(gl); x2[0] = 1.0; x2[1] = 1.0
        y2 = np.zeros(gl); y2[0] = 0.375; y2[2] = 1.0
        comp += list(x1) + list(y1) + list(x2) + list(y2)
    root = [nc]
    for (rh, rw) in spec.roots:
        root += [rh, rw, 31] + list(rng.normal(0.0, spec.root_std, size=rh * rw * 31))
    part = [len(psizes)]
    for (ph, pw) in psizes:
        part += [ph, pw, 31] + list(rng.normal(0.0, spec.part_std, size=ph * pw * 31)) + [0]
    paths = tuple(os.path.join(out_dir, f"{spec.name}_{kind}.csv") for kind in ("comp", "root", "part"))
    for p, vals in zip(paths, (comp, root, part)):
        with open(p, "w") as f:
            f.write(_fmt(vals))
    return paths


def model_paths(spec: ModelSpec, out_dir: str) -> tuple[str, str, str]:
    """Writes the model if its files are missing; returns the (comp, root, part) paths."""
    paths = tuple(os.path.join(out_dir, f"{spec.name}_{kind}.csv") for kind in ("comp", "root", "part"))
    if not all(os.path.exists(p) for p in paths):
        paths = write_model_csv(spec, out_dir)
    return paths
