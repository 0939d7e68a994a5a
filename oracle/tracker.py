"""CPU restatement of the serving tracker (geye_gb300/csrc/tracker.h, tracker.cu).

Test infrastructure only.  Parity unpinned: the reference tracks with OpenCV's
CvConDensation (CAR_TRACKING/tracking.cpp:321-850), which needs OpenCV 2.4 and
does not build here; this file restates the project's own specification
(constant velocity, Gaussian noise sigma 4 px / 1 px per frame, Philox4x32-10
draws, greedy IoU association, a particle weight of A_SCORE at the particle
plus a Gaussian corner likelihood as the reference's calc_part_likelihood adds
A_SCORE to its image likelihood (tracking.cpp:403-452), systematic
resampling) so the GPU kernels can be checked against it.

Philox4x32-10 follows Salmon, Moraes, Dror and Shaw, "Parallel random numbers:
as easy as 1, 2, 3" (SC 2011): ten rounds of two 32x32->64 multiplications by
0xD2511F53 / 0xCD9E8D57 with the Weyl key schedule 0x9E3779B9 / 0xBB67AE85.
"""
from __future__ import annotations

import numpy as np

TRACKS, PARTICLES, MAX_DET, MAX_MISSED = 32, 500, 256, 10
SIGMA_POS, SIGMA_VEL, LIKE_SCALE, ASSOC_IOU = 4.0, 1.0, 8.0, 0.3
SEED = 0x5EED5EED
M32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c = [np.asarray(x, np.uint64) & M32 for x in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(k0) & M32, np.uint64(k1) & M32
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c[0]
        p1 = np.uint64(0xCD9E8D57) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & M32
        hi1, lo1 = p1 >> np.uint64(32), p1 & M32
        c = [(hi1 ^ c[1] ^ k0) & M32, lo1, (hi0 ^ c[3] ^ k1) & M32, lo0]
        k0 = (k0 + np.uint64(0x9E3779B9)) & M32
        k1 = (k1 + np.uint64(0xBB67AE85)) & M32
    return [x.astype(np.uint32) for x in c]


def unit(x):
    return ((x >> np.uint32(8)).astype(np.float64) + 1.0) / 16777216.0


def normals4(i, draw, frame, t, k0, k1):
    r = philox4x32_10(i, np.full_like(i, draw), np.full_like(i, frame), np.full_like(i, t), k0, k1)
    a = np.sqrt(-2.0 * np.log(unit(r[0])))
    b = np.sqrt(-2.0 * np.log(unit(r[2])))
    return (a * np.cos(2 * np.pi * unit(r[1])), a * np.sin(2 * np.pi * unit(r[1])),
            b * np.cos(2 * np.pi * unit(r[3])), b * np.sin(2 * np.pi * unit(r[3])))


def keys(stream: int):
    return (SEED ^ ((stream * 0x9E3779B9) & 0xFFFFFFFF)) & 0xFFFFFFFF, (SEED >> 32) + stream


def iou(a, b):
    w = min(a[2], b[2]) - max(a[0], b[0])
    h = min(a[3], b[3]) - max(a[1], b[1])
    if w <= 0 or h <= 0:
        return 0.0
    inter = w * h
    ua = (a[2] - a[0]) * (a[3] - a[1]) + (b[2] - b[0]) * (b[3] - b[1]) - inter
    return inter / ua if ua > 0 else 0.0


def ascore_at(ascore, cx, cy):
    """Largest A_SCORE over the models at ((int)cx, (int)cy), C truncation; 0 outside the image."""
    if ascore is None:
        return 0.0
    a = np.asarray(ascore, np.float32)
    _, W, H = a.shape
    inside = (cx > -1) & (cx < W) & (cy > -1) & (cy < H)
    X = np.where(inside, np.trunc(cx), 0).astype(np.int64)
    Y = np.where(inside, np.trunc(cy), 0).astype(np.int64)
    return np.where(inside, a.max(0)[X, Y].astype(np.float64), 0.0)


class StreamTracker:
    """One stream's tracker; step(dets) runs one frame (dets: (n, 4) x1 y1 x2 y2)."""

    def __init__(self, stream: int):
        self.k0, self.k1 = keys(stream)
        self.frame = 0
        self.alive = np.zeros(TRACKS, bool)
        self.missed = np.zeros(TRACKS, int)
        self.est = np.zeros((TRACKS, 4))
        self.p = np.zeros((TRACKS, 6, PARTICLES))

    def step(self, dets: np.ndarray, ascore: np.ndarray | None = None):
        """ascore: the frame's A_SCORE maps, (n_models, W, H) indexed [m, x, y], or None."""
        dets = np.asarray(dets, np.float64)[:MAX_DET]
        nd = len(dets)
        taken = np.zeros(nd, bool)
        assign = np.full(TRACKS, -1)
        init = np.zeros(TRACKS, bool)
        for t in range(TRACKS):
            if not self.alive[t]:
                continue
            best, bi = -1.0, -1
            for d in range(nd):
                v = iou(self.est[t], dets[d])
                if not taken[d] and v >= ASSOC_IOU and v > best:
                    best, bi = v, d
            assign[t] = bi
            if bi >= 0:
                taken[bi] = True
                self.missed[t] = 0
            else:
                self.missed[t] += 1
                if self.missed[t] > MAX_MISSED:
                    self.alive[t] = False
        t = 0
        for d in range(nd):
            if taken[d]:
                continue
            while t < TRACKS and self.alive[t]:
                t += 1
            if t == TRACKS:
                break
            self.alive[t], self.missed[t], assign[t], init[t] = True, 0, d, True
            taken[d] = True
            t += 1
        self.frame += 1
        i = np.arange(PARTICLES, dtype=np.uint32)
        for t in range(TRACKS):
            if not self.alive[t]:
                continue
            if init[t]:
                d = dets[assign[t]]
                z = normals4(i, 0, self.frame, t, self.k0, self.k1)
                self.p[t] = [0.5 * (d[0] + d[2]) + SIGMA_POS * z[0], 0.5 * (d[1] + d[3]) + SIGMA_POS * z[1],
                             np.maximum(4.0, d[2] - d[0] + SIGMA_POS * z[2]),
                             np.maximum(4.0, d[3] - d[1] + SIGMA_POS * z[3]), 0 * i, 0 * i]
                self.est[t] = d
                continue
            z = normals4(i, 0, self.frame, t, self.k0, self.k1)
            zv = normals4(i, 1, self.frame, t, self.k0, self.k1)
            s = self.p[t].copy()
            s[0] += s[4] + SIGMA_POS * z[0]
            s[1] += s[5] + SIGMA_POS * z[1]
            s[2] = np.maximum(4.0, s[2] + SIGMA_POS * z[2])
            s[3] = np.maximum(4.0, s[3] + SIGMA_POS * z[3])
            s[4] += SIGMA_VEL * zv[0]
            s[5] += SIGMA_VEL * zv[1]
            b = np.stack([s[0] - 0.5 * s[2], s[1] - 0.5 * s[3], s[0] + 0.5 * s[2], s[1] + 0.5 * s[3]])
            w = np.ones(PARTICLES)
            if assign[t] >= 0:
                d = dets[assign[t]]
                w = np.exp(-((b - d[:, None]) ** 2).sum(0) / (2 * LIKE_SCALE ** 2))
            w = w + ascore_at(ascore, s[0], s[1])
            if not w.sum() > 0:
                w = np.ones(PARTICLES)
            self.est[t] = (w * b).sum(1) / w.sum()
            if assign[t] < 0:
                self.p[t] = s
                continue
            cum = np.cumsum(w)
            u0 = unit(philox4x32_10(np.uint32(0), 2, self.frame, t, self.k0, self.k1)[0]) - 1e-7
            target = (u0 + np.arange(PARTICLES)) * (cum[-1] / PARTICLES)
            idx = np.minimum(np.searchsorted(cum, target, side="left"), PARTICLES - 1)
            self.p[t] = s[:, idx]

    def boxes(self) -> np.ndarray:
        return self.est[self.alive].copy()
