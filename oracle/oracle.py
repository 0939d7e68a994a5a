"""ctypes front end of the CPU oracle (oracle/dpm_oracle.c) and of the
reference's own CPU functions built by oracle/ref/Makefile (oracle/_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py, always as the oracle results are
compared with or as the timed CPU baseline, never as the thing measured or shipped.

Array conventions follow the reference's column-major storage: a map of
d0 rows (y) by d1 columns (x) is a C-ordered numpy array of shape (d1, d0),
indexed [x, y]; features are (31, fs1, fs0); images are (3, w, h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdpm_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libgeye_ref.so")
# the reference's CAR_TRACKING sources: GEYE_REF_DIR, else a checkout named
# "reference" beside this repository; absent on machines that only run the tests
REF_SRC_DIR = os.environ.get("GEYE_REF_DIR") or os.path.normpath(
    os.path.join(HERE, "..", "..", "reference", "CAR_TRACKING"))

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compiles the oracle with its Makefile (gcc) and returns the library path."""
    src = os.path.join(HERE, "dpm_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def build_ref() -> str | None:
    """Builds oracle/_ref from the reference sources when they are present here."""
    if not os.path.isdir(REF_SRC_DIR):
        return REF_LIB_PATH if os.path.exists(REF_LIB_PATH) else None
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF_DIR={REF_SRC_DIR}"], check=True)
    return REF_LIB_PATH


class _Model(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("numcomponent", "sbin", "interval", "max_X", "max_Y", "padx", "pady",
                                         "max_scale", "im_w", "im_h", "ini")] + [
        ("ratio", C.c_float), ("ridx", _ip), ("oidx", _ip), ("offw", _fp), ("rsize", _ip), ("numpart", _ip),
        ("pidx", C.POINTER(_ip)), ("didx", C.POINTER(_ip)), ("psize", C.POINTER(_ip)),
        ("DefL", C.c_int), ("def_", _fp), ("anchor", _ip),
        ("x1", C.POINTER(_fp)), ("y1", C.POINTER(_fp)), ("x2", C.POINTER(_fp)), ("y2", C.POINTER(_fp)),
        ("NoR", C.c_int), ("root_size", _ip), ("rootfilter", C.POINTER(_fp)),
        ("NoP", C.c_int), ("part_size", _ip), ("partfilter", C.POINTER(_fp)), ("part_partner", _ip)]


class _Pyramid(C.Structure):
    _fields_ = [("LEN", C.c_int), ("feat", C.POINTER(_fp)), ("ftsize", _ip), ("imsize", _ip),
                ("scales", _fp), ("images", C.POINTER(_fp))]


class _Scores(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("LEN", "NoC", "NoP", "interval", "maxnp")] + [
        ("root", C.POINTER(_fp)), ("rsz", _ip), ("part", C.POINTER(_fp)), ("psz", _ip),
        ("M", C.POINTER(_fp)), ("Ix", C.POINTER(_ip)), ("Iy", C.POINTER(_ip)),
        ("score", C.POINTER(_fp)), ("skipped", _ip)]


class _Detection(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("D", "GL", "K", "probe_oob")] + [
        ("boxes", _fp), ("kept", _fp), ("point", _ip), ("or_point", _ip), ("type", _ip),
        ("scale", _fp), ("score", _fp)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_model_load.restype = C.POINTER(_Model)
        L.orc_model_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_float]
        L.orc_model_free.argtypes = [C.POINTER(_Model)]
        L.orc_build_pyramid.restype = C.POINTER(_Pyramid)
        L.orc_build_pyramid.argtypes = [C.POINTER(_Model), C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_free_pyramid.argtypes = [C.POINTER(_Pyramid)]
        L.orc_compute_scores.restype = C.POINTER(_Scores)
        L.orc_compute_scores.argtypes = [C.POINTER(_Model), C.POINTER(_Pyramid), C.c_int]
        L.orc_free_scores.argtypes = [C.POINTER(_Scores)]
        L.orc_boxes_from_scores.restype = _fp
        L.orc_boxes_from_scores.argtypes = [C.POINTER(_Model), C.POINTER(_Pyramid), C.POINTER(_Scores), C.c_float,
                                            C.c_void_p, _ip, _ip]
        L.orc_car_detection.argtypes = [C.POINTER(_Model), C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float,
                                        C.c_float, C.c_void_p, C.c_int, C.POINTER(_Detection)]
        L.orc_free_detection.argtypes = [C.POINTER(_Detection)]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_max_scale.argtypes = [C.POINTER(_Model), C.c_int, C.c_int]
        L.orc_ini_scales.argtypes = [C.POINTER(_Model), C.c_int, C.c_int]
        L.orc_resize_taps.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_resize.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
        L.orc_resize_dims.argtypes = [C.c_void_p, C.c_float, C.c_void_p]
        L.orc_calc_feature.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_hog_pixel.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _fp]
        L.orc_fconv.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.orc_fconv_f64.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.orc_score_f64.restype = C.c_int
        L.orc_score_f64.argtypes = [C.POINTER(_Model), C.POINTER(_Pyramid), C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
        L.orc_dt.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_void_p,
                             C.c_void_p, C.c_void_p]
        L.orc_quicksort.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.orc_nms_keep.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_void_p]
        L.orc_get_new_rects.argtypes = [C.POINTER(_Model), C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_ipl_to_float.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orc_add_part.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.orc_rootbox.argtypes = [C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_partbox.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_calc_a_score.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_float]
        L.orc_normalize_a_score.argtypes = [C.c_void_p, C.c_int, C.c_float]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Model:
    """An oracle-side model loaded from the reference CSV triple."""

    def __init__(self, comp: str, root: str, part: str, ratio: float = 1.0):
        self._p = lib().orc_model_load(comp.encode(), root.encode(), part.encode(), ratio)
        if not self._p:
            raise ValueError(f"oracle could not parse model {comp}")
        self.m = self._p.contents

    def __del__(self):
        try:
            if getattr(self, "_p", None):
                lib().orc_model_free(self._p)
        except Exception:
            pass

    def max_scale(self, width: int, height: int) -> int:
        return lib().orc_max_scale(self._p, width, height)

    @property
    def numpart(self):
        return [self.m.numpart[c] for c in range(self.m.numcomponent)]

    @property
    def gl(self) -> int:
        return (self.m.numpart[0] + 1) * 4 + 3


def ipl_to_float(frame: np.ndarray) -> np.ndarray:
    h, w, _ = frame.shape
    out = np.empty((3, w, h), dtype=np.float32)
    lib().orc_ipl_to_float(_ptr(np.ascontiguousarray(frame)), h, w, 3 * w, _ptr(out))
    return out


def resize_dims(sdims, scale):
    o = np.zeros(3, np.int32)
    lib().orc_resize_dims(_ptr(_i32(sdims)), scale, _ptr(o))
    return [int(v) for v in o]


def resize(img: np.ndarray, scale: float) -> np.ndarray:
    """img (3, w, h) column-major planes -> resized (3, w', h')."""
    c, w, h = img.shape
    sd = _i32([h, w, c])
    od = np.zeros(3, np.int32)
    lib().orc_resize_dims(_ptr(sd), scale, _ptr(od))
    out = np.zeros((c, od[1], od[0]), np.float32)
    lib().orc_resize(_ptr(_f32(img)), _ptr(sd), _ptr(od), scale, _ptr(out))
    return out


def resize_taps(sheight: int, dheight: int):
    cap = int(dheight * (sheight / dheight) + 0.99) + 2 * dheight + 8
    si = np.zeros(cap, np.int32); di = np.zeros(cap, np.int32); al = np.zeros(cap, np.float32)
    k = lib().orc_resize_taps(sheight, dheight, _ptr(si), _ptr(di), _ptr(al), cap)
    return si[:k], di[:k], al[:k]


def feature_dims(h, w, sbin):
    b0 = int(np.floor(h / sbin + 0.5)); b1 = int(np.floor(w / sbin + 0.5))
    return max(b0 - 2, 0), max(b1 - 2, 0)


def calc_feature(img: np.ndarray, sbin: int) -> np.ndarray:
    """img (3, w, h) -> features (31, fs1, fs0)."""
    _, w, h = img.shape
    f0, f1 = feature_dims(h, w, sbin)
    out = np.zeros((31, f1, f0), np.float32)
    fs = np.zeros(2, np.int32)
    lib().orc_calc_feature(_ptr(_f32(img)), h, w, sbin, _ptr(fs), _ptr(out))
    return out


def hog_bins(img: np.ndarray, sbin: int) -> np.ndarray:
    """Orientation bin of every visible pixel, (w, h) int array, -1 outside the voted area."""
    _, w, h = img.shape
    b0 = int(np.floor(h / sbin + 0.5)); b1 = int(np.floor(w / sbin + 0.5))
    out = -np.ones((w, h), np.int32)
    src = _f32(img)
    v = C.c_float()
    L = lib()
    for x in range(1, b1 * sbin - 1):
        for y in range(1, b0 * sbin - 1):
            out[x, y] = L.orc_hog_pixel(_ptr(src), h, w, x, y, C.byref(v))
    return out


def fconv(feat: np.ndarray, filt: np.ndarray) -> np.ndarray:
    """feat (31, a1, a0), filt (31, b1, b0) -> (a1-b1+1, a0-b0+1) column-major map."""
    _, a1, a0 = feat.shape
    _, b1, b0 = filt.shape
    out = np.zeros((a1 - b1 + 1, a0 - b0 + 1), np.float32)
    lib().orc_fconv(_ptr(_f32(feat)), a0, a1, _ptr(_f32(filt)), b0, b1, _ptr(out))
    return out


def fconv_f64(feat: np.ndarray, filt: np.ndarray) -> np.ndarray:
    _, a1, a0 = feat.shape
    _, b1, b0 = filt.shape
    out = np.zeros((a1 - b1 + 1, a0 - b0 + 1), np.float64)
    lib().orc_fconv_f64(_ptr(_f32(feat)), a0, a1, _ptr(_f32(filt)), b0, b1, _ptr(out))
    return out


def dt(vals: np.ndarray, ax, bx, ay, by):
    """vals (d1, d0) column-major -> (M, Ix, Iy), same shape."""
    d1, d0 = vals.shape
    M = np.zeros_like(vals, dtype=np.float32)
    Ix = np.zeros(vals.shape, np.int32); Iy = np.zeros(vals.shape, np.int32)
    dims = _i32([d0, d1])
    lib().orc_dt(_ptr(_f32(vals)), ax, bx, ay, by, _ptr(dims), _ptr(M), _ptr(Ix), _ptr(Iy))
    return M, Ix, Iy


# flip_feat (get_boxes.cpp:121-178): output channel c is input channel
# FLIP_ORD[c] - 1 with dim 1 reversed (signed orientations mirrored, the
# unsigned ones and the texture pairs swapped accordingly)
FLIP_ORD = (10, 9, 8, 7, 6, 5, 4, 3, 2, 1, 18, 17, 16, 15, 14, 13, 12, 11, 19, 27, 26, 25, 24, 23, 22, 21, 20,
            30, 31, 28, 29)


def flip_feat(feat: np.ndarray) -> np.ndarray:
    """feat (31, n1, n0) -> out[c, x, y] = feat[FLIP_ORD[c] - 1, n1 - 1 - x, y]."""
    f = _f32(feat)
    return np.ascontiguousarray(f[np.asarray(FLIP_ORD) - 1, ::-1, :])


def quicksort(vals: np.ndarray):
    a = _f32(vals).copy()
    order = np.arange(len(a), dtype=np.int32)
    if len(a):
        lib().orc_quicksort(_ptr(a), _ptr(order), 0, len(a) - 1)
    return a, order


def nms_keep(boxes: np.ndarray, overlap: float):
    """boxes [D][GL] -> (keep mask in input order, sorted order)."""
    b = _f32(boxes)
    D, GL = b.shape if b.ndim == 2 else (0, 0)
    keep = np.zeros(max(D, 1), np.int32); order = np.zeros(max(D, 1), np.int32)
    k = lib().orc_nms_keep(_ptr(b), D, GL, overlap, _ptr(keep), _ptr(order))
    return keep[:D].astype(bool), order[:D], k


class Pyramid:
    def __init__(self, model: Model, frame: np.ndarray, max_scale: int | None = None, nthreads: int = 0):
        h, w, _ = frame.shape
        self.model = model
        if max_scale is None:
            max_scale = model.max_scale(w, h)
        self.frame = np.ascontiguousarray(frame)
        self._p = lib().orc_build_pyramid(model._p, max_scale, _ptr(self.frame), h, w, 3 * w,
                                          nthreads or os.cpu_count())
        P = self._p.contents
        self.LEN = P.LEN
        self.ftsize = [(P.ftsize[2 * l], P.ftsize[2 * l + 1]) for l in range(P.LEN)]
        self.imsize = [(P.imsize[2 * l], P.imsize[2 * l + 1]) for l in range(P.LEN)]
        self.scales = np.array([P.scales[l] for l in range(P.LEN)], np.float32)

    def feat(self, l: int) -> np.ndarray:
        f0, f1 = self.ftsize[l]
        n = 31 * f0 * f1
        P = self._p.contents
        return np.ctypeslib.as_array(P.feat[l], shape=(max(n, 1),))[:n].reshape(31, f1, f0).copy()

    def image(self, l: int) -> np.ndarray:
        h, w = self.imsize[l]
        P = self._p.contents
        ll = l - self.model.m.interval if self.model.m.interval <= l < 2 * self.model.m.interval else l
        return np.ctypeslib.as_array(P.images[ll], shape=(3 * w * h,)).reshape(3, w, h).copy()

    def __del__(self):
        try:
            if getattr(self, "_p", None):
                lib().orc_free_pyramid(self._p)
        except Exception:
            pass


class Scores:
    """Per-stage outputs of the scoring driver (root/part conv, DT, final score)."""

    def __init__(self, model: Model, pyr: Pyramid, nthreads: int = 0):
        self.model, self.pyr = model, pyr
        self._p = lib().orc_compute_scores(model._p, pyr._p, nthreads or os.cpu_count())
        S = self._p.contents
        self.LEN, self.NoC, self.NoP, self.interval, self.maxnp = S.LEN, S.NoC, S.NoP, S.interval, S.maxnp
        self.skipped = [bool(S.skipped[l]) for l in range(S.LEN)]

    def _map(self, ptr, d0, d1, dtype=np.float32):
        n = d0 * d1
        if n <= 0 or not ptr:
            return np.zeros((max(d1, 0), max(d0, 0)), dtype)
        return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(d1, d0).astype(dtype, copy=True)

    def root(self, level, c):
        S = self._p.contents; i = level * self.NoC + c
        return self._map(S.root[i], S.rsz[2 * i], S.rsz[2 * i + 1])

    def part(self, L, p):
        S = self._p.contents; i = L * self.NoP + p
        return self._map(S.part[i], S.psz[2 * i], S.psz[2 * i + 1])

    def score(self, level, c):
        S = self._p.contents; i = level * self.NoC + c
        return self._map(S.score[i], S.rsz[2 * i], S.rsz[2 * i + 1])

    def dt(self, level, c, k):
        S = self._p.contents
        L = level - self.interval
        p = self.model.m.pidx[c][k]
        d0, d1 = S.psz[2 * (L * self.NoP + p)], S.psz[2 * (L * self.NoP + p) + 1]
        i = (level * self.NoC + c) * self.maxnp + k
        return (self._map(S.M[i], d0, d1), self._map(S.Ix[i], d0, d1, np.int32), self._map(S.Iy[i], d0, d1, np.int32))

    def score_f64(self, level, c):
        """(score, mag): the (level, c) score map in double precision from the same features and
        the magnitude max sum|a||b| of its root and parts, or None if the level is skipped."""
        S = self._p.contents; i = level * self.NoC + c
        r0, r1 = S.rsz[2 * i], S.rsz[2 * i + 1]
        if r0 <= 0 or r1 <= 0:
            return None
        out = np.zeros((r1, r0), np.float64)
        dims = np.zeros(2, np.int32)
        mag = np.zeros(1, np.float64)
        if lib().orc_score_f64(self.model._p, self.pyr._p, level, c, _ptr(out), _ptr(dims), _ptr(mag)) != 0:
            return None
        assert (dims[0], dims[1]) == (r0, r1)
        return out, float(mag[0])

    def boxes(self, thresh: float, a_score: np.ndarray | None = None):
        D = C.c_int(); oob = C.c_int()
        ap = _ptr(a_score) if a_score is not None else None
        bp = lib().orc_boxes_from_scores(self.model._p, self.pyr._p, self._p, thresh, ap, C.byref(D), C.byref(oob))
        GL = self.model.gl
        out = np.ctypeslib.as_array(bp, shape=(max(D.value, 1) * GL,))[:D.value * GL].reshape(D.value, GL).copy()
        lib().orc_free(C.cast(bp, C.c_void_p))
        return out, oob.value

    def __del__(self):
        try:
            if getattr(self, "_p", None):
                lib().orc_free_scores(self._p)
        except Exception:
            pass


def car_detection(model: Model, frame: np.ndarray, thresh: float = -0.5, overlap: float = 0.5,
                  a_score: np.ndarray | None = None, nthreads: int = 0) -> dict:
    """Whole path (detect + nms + get_new_rects); a_score (w, h) float32 updated in place if given."""
    h, w, _ = frame.shape
    fr = np.ascontiguousarray(frame)
    det = _Detection()
    ap = _ptr(a_score) if a_score is not None else None
    lib().orc_car_detection(model._p, _ptr(fr), h, w, 3 * w, thresh, overlap, ap, nthreads or os.cpu_count(),
                            C.byref(det))
    D, GL, K = det.D, det.GL, det.K

    def arr(p, n, dt=np.float32):
        if n <= 0:
            return np.zeros(0, dt)
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)

    out = dict(D=D, GL=GL, K=K, probe_oob=det.probe_oob,
               boxes=arr(det.boxes, D * GL).reshape(D, GL), kept=arr(det.kept, K * GL).reshape(K, GL),
               point=arr(det.point, 4 * K, np.int32).reshape(K, 4), or_point=arr(det.or_point, 4 * K, np.int32).reshape(K, 4),
               type=arr(det.type, K, np.int32), scale=arr(det.scale, K), score=arr(det.score, K))
    lib().orc_free_detection(C.byref(det))
    return out


# --------------------------------------------------------------------------
# the reference's own functions (oracle/_ref), available where the reference
# sources are present to compile them
# --------------------------------------------------------------------------
_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        path = build_ref()
        if path is None or not os.path.exists(path):
            return None
        _ref = C.CDLL(path)
    return _ref


def _R():
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference sources not available to build oracle/_ref")
    return R


def ref_resize(img: np.ndarray, scale: float) -> np.ndarray:
    c, w, h = img.shape
    sd = _i32([h, w, c])
    od = _i32(resize_dims([h, w, c], scale))
    out = np.zeros((c, od[1], od[0]), np.float32)
    _R().ref_resize(_ptr(_f32(img).copy()), _ptr(sd), _ptr(od), C.c_float(scale), _ptr(out))
    return out


def ref_flip_feat(feat: np.ndarray) -> np.ndarray:
    f = _f32(feat).copy()
    c, n1, n0 = f.shape
    out = np.zeros_like(f)
    _R().ref_flip_feat(_ptr(f), _ptr(_i32([n0, n1, c])), _ptr(out))
    return out


def ref_calc_feature(img: np.ndarray, sbin: int) -> np.ndarray:
    _, w, h = img.shape
    f0, f1 = feature_dims(h, w, sbin)
    out = np.zeros((31, f1, f0), np.float32)
    fs = np.zeros(2, np.int32)
    _R().ref_calc_feature(_ptr(_f32(img).copy()), _ptr(_i32([h, w, 3])), sbin, _ptr(fs), _ptr(out))
    return out


def ref_max_scale(numcomponent, sbin, interval, rsize, width, height) -> int:
    return _R().ref_max_scale(numcomponent, sbin, interval, _ptr(_i32(rsize)), width, height)


def ref_dt(vals: np.ndarray, ax, bx, ay, by):
    d1, d0 = vals.shape
    M = np.zeros(vals.shape, np.float32)
    Ix = np.zeros(vals.shape, np.int32); Iy = np.zeros(vals.shape, np.int32)
    f = C.c_float
    _R().ref_dt(_ptr(_f32(vals).copy()), f(ax), f(bx), f(ay), f(by), _ptr(_i32([d0, d1])), _ptr(M), _ptr(Ix), _ptr(Iy))
    return M, Ix, Iy


def ref_add_part(score: np.ndarray, M: np.ndarray, ax: int, ay: int) -> np.ndarray:
    s = _f32(score).copy()
    r1, r0 = s.shape
    p1, p0 = M.shape
    _R().ref_add_part(_ptr(s), _ptr(_f32(M).copy()), _ptr(_i32([r0, r1])), _ptr(_i32([p0, p1])), ax, ay)
    return s


def ref_rootbox(x, y, scale, rsize):
    out = np.zeros(4, np.float32)
    _R().ref_rootbox(x, y, C.c_float(scale), 0, 0, _ptr(_i32(rsize)), _ptr(out))
    return out


def ref_partbox(x, y, ax, ay, scale, psize, Ix, Iy):
    out = np.zeros(4, np.float32)
    d1, d0 = Ix.shape
    _R().ref_partbox(x, y, ax, ay, C.c_float(scale), 0, 0, _ptr(_i32(psize)), _ptr(_i32(Ix)), _ptr(_i32(Iy)),
                     _ptr(_i32([d0, d1])), _ptr(out))
    return out


def ref_calc_a_score(ac: np.ndarray, score: np.ndarray, rsize, im_h, im_w, sbin, scale):
    a = _f32(ac).copy()
    s1, s0 = score.shape
    _R().ref_calc_a_score(_ptr(a), _ptr(_f32(score).copy()), _ptr(_i32([s0, s1])), _ptr(_i32(rsize)), im_h, im_w,
                          0, 0, sbin, C.c_float(scale))
    return a


def ref_get_gmpc(score: np.ndarray, thresh: float):
    s1, s0 = score.shape
    cap = s0 * s1
    out = np.zeros(2 * max(cap, 1), np.int32)
    n = _R().ref_get_gmpc(_ptr(_f32(score).copy()), C.c_float(thresh), _ptr(_i32([s0, s1])), _ptr(out), cap)
    return out[:2 * n].reshape(n, 2)


def ref_nms_keep(boxes: np.ndarray, numpart0: int, overlap: float):
    b = _f32(boxes).copy()
    D = b.shape[0]
    keep = np.zeros(max(D, 1), np.int32)
    k = _R().ref_nms(_ptr(b), D, numpart0, C.c_float(overlap), _ptr(keep))
    return keep[:D].astype(bool), k


def ref_load_model(comp: str, root: str, part: str) -> np.ndarray:
    """Every field the reference's loader (load_model.cpp:57-530) parses from a CSV
    triple, flattened in the order ref_load_model_dump (ref_glue.cpp) writes them."""
    R = _R()
    R.ref_load_model_dump.restype = C.c_int
    R.ref_load_model_dump.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_void_p, C.c_int]
    n = R.ref_load_model_dump(comp.encode(), root.encode(), part.encode(), None, 0)
    out = np.zeros(n, np.float32)
    R.ref_load_model_dump(comp.encode(), root.encode(), part.encode(), _ptr(out), n)
    return out


def get_new_rects(model: Model, boxes: np.ndarray, width: int, height: int) -> dict:
    """The oracle's box regression (tracking.cpp:90-166) of kept records [K][GL]."""
    b = _f32(boxes)
    K = b.shape[0] if b.ndim == 2 else 0
    n = max(K, 1)
    point = np.zeros((n, 4), np.int32); or_point = np.zeros((n, 4), np.int32)
    typ = np.zeros(n, np.int32); scale = np.zeros(n, np.float32); score = np.zeros(n, np.float32)
    lib().orc_get_new_rects(model._p, _ptr(b) if K else None, K, width, height, _ptr(point), _ptr(or_point),
                            _ptr(typ), _ptr(scale), _ptr(score))
    return dict(num=K, point=point[:K], or_point=or_point[:K], type=typ[:K], scale=scale[:K], score=score[:K])


def ref_get_new_rects(comp: str, root: str, part: str, ratio: float, boxes: np.ndarray, width: int,
                      height: int) -> dict:
    """The reference's own get_new_rects (tracking.cpp:90-166) on kept records [K][GL] of the
    model its loader reads from the CSV triple."""
    R = _R()
    R.ref_get_new_rects.restype = C.c_int
    R.ref_get_new_rects.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_float, C.c_void_p, C.c_int, C.c_int,
                                    C.c_int] + [C.c_void_p] * 5
    b = _f32(boxes).copy()
    K = b.shape[0] if b.ndim == 2 else 0
    n = max(K, 1)
    point = np.zeros((n, 4), np.int32); or_point = np.zeros((n, 4), np.int32)
    typ = np.zeros(n, np.int32); scale = np.zeros(n, np.float32); score = np.zeros(n, np.float32)
    k = R.ref_get_new_rects(comp.encode(), root.encode(), part.encode(), ratio, _ptr(b), K, width, height,
                            _ptr(point), _ptr(or_point), _ptr(typ), _ptr(scale), _ptr(score))
    return dict(num=k, point=point[:k], or_point=or_point[:k], type=typ[:k], scale=scale[:k], score=score[:k])


def ref_quicksort(vals: np.ndarray):
    a = _f32(vals).copy()
    order = np.arange(len(a), dtype=np.int32)
    if len(a):
        _R().ref_quicksort(_ptr(a), _ptr(order), 0, len(a) - 1)
    return a, order
