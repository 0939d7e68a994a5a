"""Python front end of libgeye_dpm.so (the C ABI in include/geye_dpm.h).

Function names and argument meanings follow the reference's C++ entry points
so callers (and the parity tests) read like the reference:

    load_model(comp, root, part, ratio)            load_model.cpp:541
    car_detection(frame, model, thresh, A_SCORE, overlap)   detect.cpp:232
    calc_f_pyramid(frame, model)                   featurepyramid.cpp:952
    get_boxes(features, scales, FSIZE, model, A_SCORE, thresh)  get_boxes.cpp:583
    nms(boxes, overlap, numpart0)                  nms.cpp:94
    get_new_rects(frame_size, model, boxes)        tracking.cpp:90
    dt(vals, ax, bx, ay, by)                       dt.cpp:101
    fconvsMT(feat, filters)                        get_boxes_func.h:28
    resize(img, scale), calc_feature(img, sbin)    resize.cc:135, featurepyramid.cpp:263

Array layouts are the reference's column-major ones (see oracle/oracle.py for
the numpy shapes).  Every call runs on the GPU through the C ABI; there is no
CPU fallback: without the built library or a CUDA device, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

__all__ = ["GeyeError", "Context", "Model", "Server", "lib", "symbols"]

_lib = None


class GeyeError(RuntimeError):
    pass


def lib(build_if_missing: bool = True):
    """Loads libgeye_dpm.so (building it with nvcc first if it is missing)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise GeyeError(f"{path} is missing; run geye_gb300.build.build()")
            _build.build()
        L = C.CDLL(path)
        vp, ip, fp, i32 = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int
        sig = {
            "geye_ctx_create": [i32, vp, C.POINTER(vp)],
            "geye_ctx_destroy": [vp],
            "geye_ctx_set_conv_mode": [vp, i32],
            "geye_ctx_set_nms_order": [vp, i32],
            "geye_dt_tuning": [vp, vp, ip, vp],
            "geye_ctx_synchronize": [vp],
            "geye_model_load_csv": [vp, C.c_char_p, C.c_char_p, C.c_char_p, C.c_float, C.POINTER(vp)],
            "geye_model_free": [vp],
            "geye_model_info": [vp, vp],
            "geye_model_reset_scales": [vp],
            "geye_car_detection": [vp, vp, vp, i32, i32, i32, C.c_float, C.c_float, vp, vp],
            "geye_detect_multi": [vp, vp, i32, vp, i32, i32, i32, C.c_float, C.c_float, vp, vp],
            "geye_result_free": [vp],
            "geye_calc_f_pyramid": [vp, vp, vp, i32, i32, i32, ip, C.POINTER(fp), C.POINTER(ip), C.POINTER(fp)],
            "geye_get_boxes": [vp, vp, vp, vp, vp, i32, i32, i32, C.c_float, vp, C.POINTER(fp), ip],
            "geye_nms": [vp, vp, C.c_float, ip, i32, C.POINTER(fp)],
            "geye_get_new_rects": [vp, vp, vp, i32, i32, i32, vp],
            "geye_dt": [vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, vp, vp, vp, vp],
            "geye_fconv": [vp, vp, vp, vp, vp, i32, vp],
            "geye_resize": [vp, vp, vp, vp, C.c_float, vp],
            "geye_calc_feature": [vp, vp, vp, i32, vp, vp],
            "geye_flip_feat": [vp, vp, vp, C.POINTER(fp)],
            "geye_model_sym": [vp, vp, vp, vp],
            "geye_free": [vp],
            "geye_detect_device": [vp, vp, i32, vp, i32, i32, C.c_float, C.c_float],
            "geye_fetch_result": [vp, i32, vp, ip],
            "geye_ctx_enable_timing": [vp, i32],
            "geye_ctx_stage_times": [vp, vp, vp, C.POINTER(C.c_double), ip],
            "geye_debug_inject_fault": [vp, C.c_char_p, i32],
            "geye_nms_noalloc": [vp, i32, i32, C.c_float, vp, vp, vp],
            "geye_ctx_debug_counters": [vp, vp, i32],
            "geye_score_map": [vp, vp, i32, i32, vp, i32, vp],
            "geye_conv_tuning": [vp, vp, vp, vp],
            "geye_batch_create": [i32, vp, i32, i32, i32, C.POINTER(vp)],
            "geye_batch_destroy": [vp],
            "geye_batch_run": [vp, i32, vp, vp, vp, vp, C.c_float, C.c_float, vp],
            "geye_batch_stats": [vp, vp, vp],
            "geye_detect_submit": [vp, vp, i32, vp, i32, i32, i32, C.c_float, C.c_float],
            "geye_detect_query": [vp],
            "geye_detect_collect": [vp, vp],
            "geye_server_create": [i32, vp, i32, i32, C.c_size_t, i32, C.c_float, C.c_float, i32, C.POINTER(vp)],
            "geye_server_destroy": [vp],
            "geye_server_submit": [vp, i32, vp, i32, i32, i32, C.POINTER(C.c_longlong)],
            "geye_server_poll": [vp, i32, vp, vp, ip],
            "geye_server_drain": [vp],
            "geye_server_set_admission": [vp, i32, C.c_longlong],
            "geye_server_stats": [vp, vp],
            "geye_server_tracks": [vp, i32, i32, vp, ip],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.geye_last_error.restype = C.c_char_p
        L.geye_last_error.argtypes = []
        L.geye_version.restype = C.c_char_p
        L.geye_version.argtypes = []
        _lib = L
    return _lib


def symbols() -> list[str]:
    """Entry points declared in include/geye_dpm.h."""
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "geye_dpm.h")
    pat = r"^\s*(?:geye_status|const char \*|void)\s*\**\s*(geye_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(pat, open(hdr).read(), flags=re.M)))


class _Result(C.Structure):
    _fields_ = [("num", C.c_int), ("point", C.POINTER(C.c_int)), ("or_point", C.POINTER(C.c_int)),
                ("type", C.POINTER(C.c_int)), ("scale", C.POINTER(C.c_float)), ("score", C.POINTER(C.c_float))]


def _check(status: int, what: str):
    if status != 0:
        msg = lib().geye_last_error()
        raise GeyeError(f"{what} failed (status {status}): {msg.decode() if msg else ''}")


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _result_to_dict(r: _Result) -> dict:
    n = r.num

    def arr(ptr, k, dt):
        if n <= 0:
            return np.zeros((0,) if k == 1 else (0, k), dt)
        a = np.ctypeslib.as_array(ptr, shape=(n * k,)).astype(dt, copy=True)
        return a if k == 1 else a.reshape(n, k)

    out = dict(num=n, point=arr(r.point, 4, np.int32), or_point=arr(r.or_point, 4, np.int32),
               type=arr(r.type, 1, np.int32), scale=arr(r.scale, 1, np.float32), score=arr(r.score, 1, np.float32))
    lib().geye_result_free(C.byref(r))
    return out


CONV_FP32, CONV_BF16, CONV_FP8 = 0, 1, 2
# whole-path NMS order (geye_ctx_set_nms_order)
NMS_ORDER_KEY, NMS_ORDER_QUICKSORT = 0, 1


class Context:
    """One device and one stream (replaces init_cuda / clean_cuda, GPU_init.cpp:50-356)."""

    def __init__(self, device: int = 0, stream: int | None = None, conv: int = CONV_FP32):
        h = C.c_void_p()
        _check(lib().geye_ctx_create(device, C.c_void_p(stream) if stream else None, C.byref(h)), "geye_ctx_create")
        self.h = h
        if conv != CONV_FP32:
            self.set_conv_mode(conv)

    def close(self):
        if getattr(self, "h", None):
            lib().geye_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_conv_mode(self, mode: int):
        _check(lib().geye_ctx_set_conv_mode(self.h, mode), "set_conv_mode")

    def set_nms_order(self, order: int):
        """NMS_ORDER_KEY (default: score order, the quicksort's order only for a model
        that needs it) or NMS_ORDER_QUICKSORT (the quicksort's order always)."""
        _check(lib().geye_ctx_set_nms_order(self.h, order), "set_nms_order")

    def synchronize(self):
        _check(lib().geye_ctx_synchronize(self.h), "synchronize")

    # ---- whole path -------------------------------------------------------
    def car_detection(self, frame: np.ndarray, model: "Model", thresh: float = -0.5, A_SCORE: np.ndarray | None = None,
                      overlap: float = 0.5) -> dict:
        """frame (h, w, 3) uint8 BGR; A_SCORE (w, h) float32 updated in place if given."""
        fr = np.ascontiguousarray(frame, dtype=np.uint8)
        h, w, _ = fr.shape
        r = _Result()
        a = _p(A_SCORE) if A_SCORE is not None else None
        if A_SCORE is not None:
            assert A_SCORE.dtype == np.float32 and A_SCORE.flags.c_contiguous and A_SCORE.size == w * h
        _check(lib().geye_car_detection(self.h, model.h, _p(fr), w, h, 3 * w, thresh, overlap, a, C.byref(r)),
               "car_detection")
        return _result_to_dict(r)

    def detect_multi(self, frame: np.ndarray, models: list, thresh: float = -0.5, overlap: float = 0.5,
                     A_SCOREs: list | None = None) -> list:
        fr = np.ascontiguousarray(frame, dtype=np.uint8)
        h, w, _ = fr.shape
        n = len(models)
        arr = (C.c_void_p * n)(*[m.h for m in models])
        res = (_Result * n)()
        ap = None
        if A_SCOREs is not None:
            ap = (C.c_void_p * n)(*[_p(a) for a in A_SCOREs])
        _check(lib().geye_detect_multi(self.h, arr, n, _p(fr), w, h, 3 * w, thresh, overlap, ap, res), "detect_multi")
        return [_result_to_dict(res[i]) for i in range(n)]

    # ---- asynchronous submission ------------------------------------------
    def detect_submit(self, frame: np.ndarray, models: list, thresh: float = -0.5, overlap: float = 0.5):
        fr = np.ascontiguousarray(frame, dtype=np.uint8)
        h, w, _ = fr.shape
        arr = (C.c_void_p * len(models))(*[m.h for m in models])
        _check(lib().geye_detect_submit(self.h, arr, len(models), _p(fr), w, h, 3 * w, thresh, overlap),
               "detect_submit")
        self._submitted = len(models)

    def detect_done(self) -> bool:
        st = lib().geye_detect_query(self.h)
        if st == 8:   # GEYE_BUSY
            return False
        _check(st, "detect_query")
        return True

    def detect_collect(self) -> list:
        n = getattr(self, "_submitted", 0)
        res = (_Result * max(n, 1))()
        _check(lib().geye_detect_collect(self.h, res), "detect_collect")
        return [_result_to_dict(res[i]) for i in range(n)]

    # ---- stages -----------------------------------------------------------
    def calc_f_pyramid(self, frame: np.ndarray, model: "Model"):
        """-> (list of (31, fs1, fs0) features, FTSIZE (LEN, 2), scales (LEN,))."""
        fr = np.ascontiguousarray(frame, dtype=np.uint8)
        h, w, _ = fr.shape
        n = C.c_int()
        fp, ip, sp = C.POINTER(C.c_float)(), C.POINTER(C.c_int)(), C.POINTER(C.c_float)()
        _check(lib().geye_calc_f_pyramid(self.h, model.h, _p(fr), w, h, 3 * w, C.byref(n), C.byref(fp), C.byref(ip),
                                         C.byref(sp)), "calc_f_pyramid")
        L = n.value
        fs = np.ctypeslib.as_array(ip, shape=(2 * L,)).reshape(L, 2).copy()
        sc = np.ctypeslib.as_array(sp, shape=(L,)).copy()
        total = int(sum(31 * a * b for a, b in fs))
        flat = np.ctypeslib.as_array(fp, shape=(max(total, 1),))[:total].copy()
        for q in (fp, ip, sp):
            lib().geye_free(C.cast(q, C.c_void_p))
        feats, o = [], 0
        for a, b in fs:
            k = 31 * a * b
            feats.append(flat[o:o + k].reshape(31, b, a))
            o += k
        return feats, fs, sc

    def get_boxes(self, feats, scales, ftsize, model: "Model", thresh: float = -0.5, A_SCORE=None,
                  img_size: tuple | None = None) -> np.ndarray:
        """feats: list of (31, fs1, fs0); returns boxes [D][GL]."""
        flat = np.ascontiguousarray(np.concatenate([np.asarray(f, np.float32).ravel() for f in feats]))
        sc = np.ascontiguousarray(scales, np.float32)
        fs = np.ascontiguousarray(ftsize, np.int32).ravel()
        w, h = img_size if img_size else (0, 0)
        bp = C.POINTER(C.c_float)()
        d = C.c_int()
        _check(lib().geye_get_boxes(self.h, model.h, _p(flat), _p(sc), _p(fs), len(feats), w, h, thresh,
                                    _p(A_SCORE) if A_SCORE is not None else None, C.byref(bp), C.byref(d)),
               "get_boxes")
        GL = model.gl
        D = d.value
        out = np.ctypeslib.as_array(bp, shape=(max(D, 1) * GL,))[:D * GL].reshape(D, GL).copy()
        lib().geye_free(C.cast(bp, C.c_void_p))
        return out

    def nms(self, boxes: np.ndarray, overlap: float, numpart0: int) -> np.ndarray:
        b = np.ascontiguousarray(boxes, np.float32)
        num = C.c_int(b.shape[0] if b.ndim == 2 else 0)
        GL = (numpart0 + 1) * 4 + 3
        op = C.POINTER(C.c_float)()
        _check(lib().geye_nms(self.h, _p(b) if b.size else None, overlap, C.byref(num), numpart0, C.byref(op)), "nms")
        K = num.value
        if not op:
            return np.zeros((0, GL), np.float32)
        out = np.ctypeslib.as_array(op, shape=(max(K, 1) * GL,))[:K * GL].reshape(K, GL).copy()
        lib().geye_free(C.cast(op, C.c_void_p))
        return out

    def get_new_rects(self, img_size: tuple, model: "Model", boxes: np.ndarray) -> dict:
        b = np.ascontiguousarray(boxes, np.float32)
        r = _Result()
        w, h = img_size
        _check(lib().geye_get_new_rects(self.h, model.h, _p(b) if b.size else None, b.shape[0], w, h, C.byref(r)),
               "get_new_rects")
        return _result_to_dict(r)

    def dt(self, vals: np.ndarray, ax, bx, ay, by):
        v = np.ascontiguousarray(vals, np.float32)
        d1, d0 = v.shape
        M = np.zeros_like(v)
        Ix = np.zeros(v.shape, np.int32)
        Iy = np.zeros(v.shape, np.int32)
        dims = np.array([d0, d1], np.int32)
        _check(lib().geye_dt(self.h, _p(v), ax, bx, ay, by, _p(dims), _p(M), _p(Ix), _p(Iy)), "dt")
        return M, Ix, Iy

    def fconvsMT(self, feat: np.ndarray, filters: list) -> list:
        f = np.ascontiguousarray(feat, np.float32)
        _, a1, a0 = f.shape
        fl = [np.ascontiguousarray(x, np.float32) for x in filters]
        ptrs = (C.c_void_p * len(fl))(*[x.ctypes.data for x in fl])
        bd = np.array([[x.shape[2], x.shape[1]] for x in fl], np.int32).ravel()
        sizes = [(a1 - x.shape[1] + 1, a0 - x.shape[2] + 1) for x in fl]
        out = np.zeros(sum(p * q for p, q in sizes), np.float32)
        _check(lib().geye_fconv(self.h, _p(f), _p(np.array([a0, a1], np.int32)), ptrs, _p(bd), len(fl), _p(out)),
               "fconv")
        res, o = [], 0
        for p, q in sizes:
            res.append(out[o:o + p * q].reshape(p, q))
            o += p * q
        return res

    def resize(self, img: np.ndarray, scale: float) -> np.ndarray:
        a = np.ascontiguousarray(img, np.float32)
        c, w, h = a.shape
        sd = np.array([h, w, c], np.int32)
        od = np.zeros(3, np.int32)
        if scale == 1.0:
            return a.copy()
        oh, ow = int(np.float32(h) * np.float32(scale) + 0.5), int(np.float32(w) * np.float32(scale) + 0.5)
        out = np.zeros((c, ow, oh), np.float32)
        _check(lib().geye_resize(self.h, _p(a), _p(sd), _p(od), scale, _p(out)), "resize")
        assert (od[0], od[1]) == (oh, ow)
        return out

    def calc_feature(self, img: np.ndarray, sbin: int) -> np.ndarray:
        a = np.ascontiguousarray(img, np.float32)
        _, w, h = a.shape
        b0, b1 = int(np.floor(h / sbin + 0.5)), int(np.floor(w / sbin + 0.5))
        f0, f1 = max(b0 - 2, 0), max(b1 - 2, 0)
        out = np.zeros((31, f1, f0), np.float32)
        fs = np.zeros(2, np.int32)
        _check(lib().geye_calc_feature(self.h, _p(a), _p(np.array([h, w, 3], np.int32)), sbin, _p(fs), _p(out)),
               "calc_feature")
        return out

    def flip_feat(self, feat: np.ndarray) -> np.ndarray:
        """flip_feat (get_boxes.cpp:121-178): feat (31, n1, n0) -> mirrored along n1, channels reordered."""
        f = np.ascontiguousarray(feat, np.float32)
        c, n1, n0 = f.shape
        op = C.POINTER(C.c_float)()
        _check(lib().geye_flip_feat(self.h, _p(f), _p(np.array([n0, n1, c], np.int32)), C.byref(op)), "flip_feat")
        n = c * n1 * n0
        out = np.ctypeslib.as_array(op, shape=(max(n, 1),))[:n].reshape(c, n1, n0).copy()
        lib().geye_free(C.cast(op, C.c_void_p))
        return out

    # ---- device-resident path ---------------------------------------------
    def detect_device(self, d_bgr_ptr: int, width: int, height: int, models: list, thresh: float = -0.5,
                      overlap: float = 0.5):
        arr = (C.c_void_p * len(models))(*[m.h for m in models])
        _check(lib().geye_detect_device(self.h, arr, len(models), C.c_void_p(d_bgr_ptr), width, height, thresh,
                                        overlap), "detect_device")

    def fetch_result(self, model_index: int = 0):
        r = _Result()
        D = C.c_int()
        _check(lib().geye_fetch_result(self.h, model_index, C.byref(r), C.byref(D)), "fetch_result")
        out = _result_to_dict(r)
        out["D"] = D.value
        return out

    def enable_timing(self, on: bool = True):
        _check(lib().geye_ctx_enable_timing(self.h, 1 if on else 0), "enable_timing")

    def stage_times(self) -> dict:
        ms = (C.c_float * 7)()
        by = (C.c_double * 7)()
        fl = C.c_double()
        nl = C.c_int()
        _check(lib().geye_ctx_stage_times(self.h, ms, by, C.byref(fl), C.byref(nl)), "stage_times")
        names = ["pyramid", "hog", "conv", "dt", "score", "nms", "total"]
        return dict(ms={n: ms[i] for i, n in enumerate(names)}, bytes={n: by[i] for i, n in enumerate(names)},
                    conv_flops=fl.value, launches=nl.value)

    def debug_counters(self, n: int = 16) -> list:
        out = (C.c_longlong * n)()
        _check(lib().geye_ctx_debug_counters(self.h, out, n), "debug_counters")
        return list(out)

    def score_map(self, model: "Model", level: int, comp: int) -> np.ndarray:
        """Score map of (level, component) from the last whole-path run, shape (r1, r0)
        (column-major r0 x r1 as the reference stores it)."""
        dims = np.zeros(2, np.int32)
        _check(lib().geye_score_map(self.h, model.h, level, comp, None, 0, _p(dims)), "score_map")
        out = np.zeros((int(dims[1]), int(dims[0])), np.float32)
        _check(lib().geye_score_map(self.h, model.h, level, comp, _p(out), out.size, _p(dims)), "score_map")
        return out

    def conv_tuning(self, model: "Model") -> dict:
        """Tile shape the tensor-core convolution's autotuner chose for the model in the last run's plan
        (tiles_per_cta 0: the persistent form, one CTA per SM with the filter bank resident)."""
        shape = np.zeros(3, np.int32)
        ms = np.zeros(1, np.float32)
        _check(lib().geye_conv_tuning(self.h, model.h, _p(shape), _p(ms)), "conv_tuning")
        return {"tiles_per_cta": int(shape[0]), "smem_kb": int(shape[1]), "ctas": int(shape[2]), "ms": float(ms[0])}

    def dt_tuning(self, model: "Model") -> dict:
        """DT tile size (outputs per block) the plan of the last run chose for the model, and the
        timed launch of each candidate (1024, 2048, 4096 outputs per block; zeros before tuning)."""
        elems = C.c_int()
        ms = np.zeros(3, np.float32)
        _check(lib().geye_dt_tuning(self.h, model.h, C.byref(elems), _p(ms)), "dt_tuning")
        return {"elems": elems.value, "ms": ms.tolist()}

    def inject_fault(self, op: str | None, nth: int):
        _check(lib().geye_debug_inject_fault(self.h, op.encode() if op else None, nth), "inject_fault")


class _Served(C.Structure):
    _fields_ = [("ticket", C.c_longlong), ("stream", C.c_int), ("n_tracks", C.c_int), ("queued_ns", C.c_longlong),
                ("latency_ns", C.c_longlong), ("dropped", C.c_int), ("reserved", C.c_int)]


class Server:
    """Multi-stream detection server (geye_server_*): frames are admitted into
    slots as they arrive and overlap on the GPU; optional per-stream trackers."""

    def __init__(self, models: list, conv: int = CONV_BF16, hbm_budget: int = 40 << 30, max_slots: int = 16,
                 thresh: float = -0.5, overlap: float = 0.5, track: bool = False, device: int = 0):
        h = C.c_void_p()
        arr = (C.c_void_p * len(models))(*[m.h for m in models])
        _check(lib().geye_server_create(device, arr, len(models), conv, hbm_budget, max_slots, thresh, overlap,
                                        1 if track else 0, C.byref(h)), "server_create")
        self.h = h
        self.n_models = len(models)

    def submit(self, stream: int, frame: np.ndarray) -> int:
        fr = np.ascontiguousarray(frame, dtype=np.uint8)
        hh, w, _ = fr.shape
        t = C.c_longlong()
        _check(lib().geye_server_submit(self.h, stream, _p(fr), w, hh, 3 * w, C.byref(t)), "server_submit")
        return t.value

    def poll(self, max_results: int = 256, with_results: bool = True) -> list:
        info = (_Served * max_results)()
        res = (_Result * (max_results * self.n_models))() if with_results else None
        n = C.c_int()
        _check(lib().geye_server_poll(self.h, max_results, info, res, C.byref(n)), "server_poll")
        out = []
        for i in range(n.value):
            d = dict(ticket=info[i].ticket, stream=info[i].stream, n_tracks=info[i].n_tracks,
                     queued_ns=info[i].queued_ns, latency_ns=info[i].latency_ns, dropped=bool(info[i].dropped))
            if with_results:
                d["results"] = [_result_to_dict(res[i * self.n_models + m]) for m in range(self.n_models)]
            out.append(d)
        return out

    def drain(self):
        _check(lib().geye_server_drain(self.h), "server_drain")

    def set_admission(self, max_queued_per_stream: int = 0, max_wait_ms: float = 0.0):
        """Per-stream queue cap (a newer frame drops the stream's oldest waiting one)
        and the longest a frame may wait for a slot; 0 = no limit."""
        _check(lib().geye_server_set_admission(self.h, max_queued_per_stream, int(max_wait_ms * 1e6)),
               "server_set_admission")

    def stats(self) -> dict:
        o = np.zeros(8, np.int64)
        _check(lib().geye_server_stats(self.h, _p(o)), "server_stats")
        keys = ["slots", "busy", "queued", "finished", "bytes_held", "completed", "tracked_streams", "dropped"]
        return dict(zip(keys, [int(v) for v in o]))

    def tracks(self, stream: int, max_tracks: int = 64) -> np.ndarray:
        b = np.zeros((max_tracks, 4), np.float32)
        n = C.c_int()
        _check(lib().geye_server_tracks(self.h, stream, max_tracks, _p(b), C.byref(n)), "server_tracks")
        return b[:min(n.value, max_tracks)].copy()

    def close(self):
        if getattr(self, "h", None):
            lib().geye_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Several frames of any sizes as one CUDA graph (geye_batch_*): one lane per
    frame, the lanes parallel branches of one graph; results per frame and model."""

    def __init__(self, models: list, conv: int = CONV_FP32, max_frames: int = 32, device: int = 0):
        arr = (C.c_void_p * len(models))(*[m.h for m in models])
        h = C.c_void_p()
        _check(lib().geye_batch_create(device, arr, len(models), conv, max_frames, C.byref(h)), "batch_create")
        self.h = h.value
        self.n_models = len(models)
        self.models = models

    def run(self, frames: list, thresh: float = -0.5, overlap: float = 0.5) -> list:
        fr = [np.ascontiguousarray(f, dtype=np.uint8) for f in frames]
        n = len(fr)
        ptrs = (C.c_void_p * n)(*[f.ctypes.data for f in fr])
        w = np.array([f.shape[1] for f in fr], np.int32)
        h = np.array([f.shape[0] for f in fr], np.int32)
        st = 3 * w
        res = (_Result * (n * self.n_models))()
        _check(lib().geye_batch_run(self.h, n, ptrs, _p(w), _p(h), _p(st), thresh, overlap, res), "batch_run")
        return [[_result_to_dict(res[i * self.n_models + m]) for m in range(self.n_models)] for i in range(n)]

    def stats(self) -> dict:
        o = np.zeros(4, np.int32)
        ms = np.zeros(1, np.float32)
        _check(lib().geye_batch_stats(self.h, _p(o), _p(ms)), "batch_stats")
        return {"lanes": int(o[0]), "graphs": int(o[1]), "kernels": int(o[2]), "last_ms": float(ms[0])}

    def close(self):
        if getattr(self, "h", None):
            lib().geye_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Model:
    """A DPM model on the device (replaces load_model / free_model)."""

    def __init__(self, ctx: Context, comp: str, root: str, part: str, ratio: float = 1.0):
        h = C.c_void_p()
        _check(lib().geye_model_load_csv(ctx.h, comp.encode(), root.encode(), part.encode(), ratio, C.byref(h)),
               "model_load_csv")
        self.h = h
        self.ctx = ctx
        info = np.zeros(8, np.int32)
        _check(lib().geye_model_info(h, _p(info)), "model_info")
        self.numcomponent, self.sbin, self.interval, self.numpart0, self.gl, self.NoR, self.NoP, _ = [int(v) for v in info]

    def info(self) -> dict:
        info = np.zeros(8, np.int32)
        _check(lib().geye_model_info(self.h, _p(info)), "model_info")
        keys = ["numcomponent", "sbin", "interval", "numpart0", "GL", "NoR", "NoP", "max_scale"]
        return dict(zip(keys, [int(v) for v in info]))

    def reset_scales(self):
        _check(lib().geye_model_reset_scales(self.h), "reset_scales")

    def sym(self) -> dict:
        """Symmetric information (load_model.cpp:279-373, 420-524): rootsym, part_partner, part_sym."""
        rs = np.zeros(max(self.NoR, 1), np.int32)
        pp = np.zeros(max(self.NoP, 1), np.int32)
        ps = np.zeros(max(self.NoP, 1), np.int32)
        _check(lib().geye_model_sym(self.h, _p(rs), _p(pp), _p(ps)), "model_sym")
        return {"rootsym": rs[:self.NoR], "part_partner": pp[:self.NoP], "part_sym": ps[:self.NoP]}

    def close(self):
        if getattr(self, "h", None):
            lib().geye_model_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
