"""The reference's own test data on the CPU: the PNG reader, the trained car
and person models as the reference's loader parses them, and the oracle's
detections on the 21 real frames (tests/golden/real_*.npz, written by
tests/golden/make_real_golden.py).  The checks against the reference's sources
run only where they are present; the rest run on any machine."""
import os
import struct
import sys
import tempfile
import zlib

import numpy as np
import pytest

from geye_gb300 import png
from oracle import oracle as O

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import real_data as RD  # noqa: E402

needs_ref = pytest.mark.skipif(O.ref_lib() is None, reason="reference sources not present to build oracle/_ref")


# ---------------------------------------------------------------------------
# PNG reader
# ---------------------------------------------------------------------------
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _encode(img: np.ndarray, filters) -> bytes:
    """A PNG encoder written from the specification's forward filters, one filter type per row."""
    h, w, ch = img.shape
    ctype = {1: 0, 3: 2, 4: 6}[ch]
    raw = bytearray()
    prev = [0] * (w * ch)
    for y in range(h):
        ft = filters[y % len(filters)]
        cur = img[y].reshape(-1).tolist()
        out = []
        for i, x in enumerate(cur):
            a = cur[i - ch] if i >= ch else 0
            b = prev[i]
            c = prev[i - ch] if i >= ch else 0
            pred = (0, a, b, (a + b) >> 1, _paeth(a, b, c))[ft]
            out.append((x - pred) & 0xFF)
        raw += bytes([ft]) + bytes(out)
        prev = cur

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)
    z = zlib.compress(bytes(raw))
    # IDAT split in two chunks: the reader must join them
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", z[:len(z) // 2])
            + chunk(b"IDAT", z[len(z) // 2:]) + chunk(b"IEND", b""))


@pytest.mark.parametrize("ch", [1, 3, 4])
def test_png_every_row_filter_round_trips(ch):
    rng = np.random.default_rng(ch)
    img = rng.integers(0, 256, size=(23, 17, ch)).astype(np.uint8)
    img[5:12, 3:9] = 200           # flat areas: zero residuals
    data = _encode(img, [0, 1, 2, 3, 4])
    assert np.array_equal(png.decode(data), img)


def test_png_load_bgr_swaps_to_iplimage_order(tmp_path):
    img = np.random.default_rng(7).integers(0, 256, size=(9, 11, 3)).astype(np.uint8)
    p = tmp_path / "f.png"
    p.write_bytes(_encode(img, [4, 3]))
    bgr = png.load_bgr(str(p))
    assert bgr.flags["C_CONTIGUOUS"] and np.array_equal(bgr, img[:, :, ::-1])


def test_png_rejects_damaged_and_unsupported_files():
    img = np.zeros((4, 5, 3), np.uint8)
    data = bytearray(_encode(img, [1]))
    with pytest.raises(png.PngError):
        png.decode(b"GIF89a" + bytes(data[6:]))
    bad = bytearray(data)
    bad[40] ^= 0xFF                 # a byte inside IHDR/IDAT: CRC mismatch
    with pytest.raises(png.PngError):
        png.decode(bytes(bad))
    ihdr16 = data[:8] + struct.pack(">I", 13) + b"IHDR" + struct.pack(">IIBBBBB", 5, 4, 16, 2, 0, 0, 0)
    ihdr16 += struct.pack(">I", zlib.crc32(b"IHDR" + ihdr16[16:]) & 0xFFFFFFFF)
    with pytest.raises(png.PngError):
        png.decode(bytes(ihdr16 + data[33:]))


@needs_ref
def test_png_reference_frames_decode_to_the_fixture():
    frames = RD.load_frames()
    for i in (0, 7, 20):
        f = png.load_bgr(os.path.join(O.REF_SRC_DIR, "Test_Images", "org_image", f"{i}.png"))
        assert f.shape == (480, 640, 3) and np.array_equal(f, frames[i]), i


def test_real_frames_fixture_shape():
    frames = RD.load_frames()
    assert frames.shape == (21, 480, 640, 3) and frames.dtype == np.uint8
    # natural images: neighbouring pixels are close (a wrong row filter leaves noise)
    d = np.abs(np.diff(frames.astype(np.int16), axis=2)).mean()
    assert d < 12, d


# ---------------------------------------------------------------------------
# trained models
# ---------------------------------------------------------------------------
@needs_ref
@pytest.mark.parametrize("name", RD.MODEL_NAMES)
def test_reference_loader_fields_match_fixture(name):
    paths = [os.path.join(O.REF_SRC_DIR, f"{name}_{k}.csv") for k in ("comp", "root", "part")]
    got = O.ref_load_model(*paths)
    want = RD.model_dump(name)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    with tempfile.TemporaryDirectory() as d:
        again = O.ref_load_model(*RD.write_model_csv(want, d, name))
    assert np.array_equal(again.view(np.uint32), want.view(np.uint32))


def _oracle_fields(m: O.Model) -> dict:
    M = m.m
    f = dict(numcomponent=M.numcomponent, sbin=M.sbin, interval=M.interval, max_Y=M.max_Y, max_X=M.max_X)
    comps = []
    for c in range(M.numcomponent):
        np_ = M.numpart[c]
        gl = 1 + 2 * (1 + np_)
        comps.append(dict(ridx=M.ridx[c], oidx=M.oidx[c], offw=np.float32(M.offw[c]),
                          rsize=[M.rsize[2 * c], M.rsize[2 * c + 1]], numpart=np_,
                          parts=[dict(pidx=M.pidx[c][k], didx=M.didx[c][k],
                                      psize=[M.psize[c][2 * k], M.psize[c][2 * k + 1]]) for k in range(np_)],
                          **{k: np.array([getattr(M, k)[c][j] for j in range(gl)], np.float32)
                             for k in ("x1", "y1", "x2", "y2")}))
    f["comps"] = comps
    f["def"] = np.array([M.def_[i] for i in range(4 * M.DefL)], np.float32).reshape(-1, 4)
    f["anchor"] = np.array([M.anchor[i] for i in range(2 * M.DefL)], np.int32).reshape(-1, 2)
    f["roots"] = [dict(size=[M.root_size[3 * r + i] for i in range(3)],
                       w=np.array([M.rootfilter[r][i] for i in range(M.root_size[3 * r] * M.root_size[3 * r + 1] * 31)],
                                  np.float32)) for r in range(M.NoR)]
    f["parts"] = [dict(size=[M.part_size[3 * p + i] for i in range(3)], partner=M.part_partner[p],
                       w=np.array([M.partfilter[p][i] for i in range(M.part_size[3 * p] * M.part_size[3 * p + 1] * 31)],
                                  np.float32)) for p in range(M.NoP)]
    return f


@pytest.mark.parametrize("name", RD.MODEL_NAMES)
def test_oracle_loader_reads_the_reference_loaders_fields(name, tmp_path):
    """The oracle's CSV parser against the reference loader's parse of the trained models."""
    want = RD.parse_dump(RD.model_dump(name))
    got = _oracle_fields(O.Model(*RD.write_model_csv(RD.model_dump(name), str(tmp_path), name)))
    for k in ("numcomponent", "sbin", "interval", "max_Y", "max_X"):
        assert got[k] == want[k], k
    for cg, cw in zip(got["comps"], want["comps"]):
        for k in ("ridx", "oidx", "rsize", "numpart", "parts"):
            assert cg[k] == cw[k], k
        assert cg["offw"].view(np.uint32) == cw["offw"].view(np.uint32)
        for k in ("x1", "y1", "x2", "y2"):
            assert np.array_equal(cg[k].view(np.uint32), cw[k].view(np.uint32)), k
    assert np.array_equal(got["def"].view(np.uint32), want["def"].view(np.uint32))
    assert np.array_equal(got["anchor"], want["anchor"])
    assert len(got["roots"]) == len(want["roots"]) and len(got["parts"]) == len(want["parts"])
    for g, w in zip(got["roots"] + got["parts"], want["roots"] + want["parts"]):
        assert g["size"] == w["size"] and np.array_equal(g["w"].view(np.uint32), w["w"].view(np.uint32))
    for g, w in zip(got["parts"], want["parts"]):
        assert g["partner"] == w["partner"]


def test_trained_models_shape():
    """What the pipeline has to cover: non-square parts of several sizes per model."""
    for name in RD.MODEL_NAMES:
        f = RD.parse_dump(RD.model_dump(name))
        assert f["numcomponent"] == 2 and f["sbin"] == 8 and f["interval"] == 10
        sizes = {tuple(p["size"][:2]) for p in f["parts"]}
        assert len(sizes) >= 3 and any(a != b for a, b in sizes), sizes
        assert all(c["numpart"] == f["comps"][0]["numpart"] for c in f["comps"])


# ---------------------------------------------------------------------------
# the oracle on the real frames
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def real_models(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("real_models"))
    return {n: O.Model(*RD.write_model_csv(RD.model_dump(n), d, n), RD.RATIO) for n in RD.MODEL_NAMES}


@pytest.mark.parametrize("name,frame", [("car", 5), ("car", 13), ("car", 20), ("person", 1), ("person", 6)])
def test_oracle_reproduces_real_frame_fixture(real_models, name, frame):
    frames = RD.load_frames()
    E = RD.expected(name, frame)
    a = np.full((640, 480), -100, np.float32)
    r = O.car_detection(real_models[name], frames[frame], RD.THRESH, RD.OVERLAP, a_score=a)
    assert r["D"] == int(E["D"])
    for k in ("kept", "scale", "score"):
        assert np.array_equal(r[k].view(np.uint32), E[k].view(np.uint32)), k
    for k in ("point", "or_point", "type"):
        assert np.array_equal(r[k], E[k]), k
    assert RD.float_digest(a) == E["a_score_sha256"].tobytes()


@needs_ref
def test_oracle_stages_on_a_real_frame_match_reference_functions(real_models):
    """Frame 0 through the reference's own resize, calc_feature and dt, level by level."""
    m = real_models["car"]
    fr = RD.load_frames()[0]
    P = O.Pyramid(m, fr)
    img0 = O.ipl_to_float(fr)
    sc = np.float32(2.0 ** (1.0 / 10))
    imgs = {ii: O.ref_resize(img0, float(np.float32(1.0 / (float(sc) ** ii)))) for ii in range(10)}
    for ii in range(10):
        cur = imgs[ii]
        for jj in range(ii + 10, P.LEN - 10, 10):
            cur = O.ref_resize(cur, 0.5)
            imgs[jj + 10] = cur
    for lv in (0, 5, 10, 17, 20, 34):
        im = imgs[lv] if lv < 10 or lv >= 20 else imgs[lv - 10]
        f = O.ref_calc_feature(im, 4 if lv < 10 else 8)
        assert np.array_equal(P.feat(lv).view(np.int32), f.view(np.int32)), f"level {lv}"
    S = O.Scores(m, P)
    for lv in (10, 15, 22):
        for c in range(S.NoC):
            for k in range(m.numpart[c]):
                p = m.m.pidx[c][k]
                di = m.m.didx[c][k]
                part = S.part(lv - S.interval, p)
                coef = [m.m.def_[4 * di + j] for j in range(4)]
                M, Ix, Iy = O.ref_dt(-part, *coef)
                gM, gIx, gIy = S.dt(lv, c, k)
                assert np.array_equal(gM.view(np.int32), M.view(np.int32)) and np.array_equal(gIx, Ix) \
                    and np.array_equal(gIy, Iy), (lv, c, k)


# ---------------------------------------------------------------------------
# get_new_rects against the reference's own function
# ---------------------------------------------------------------------------
def _same_rects(got, want, where):
    assert got["num"] == len(want["score"]), where
    for k in ("point", "or_point", "type"):
        assert np.array_equal(got[k], want[k]), (where, k)
    for k in ("scale", "score"):
        assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), (where, k)


@pytest.mark.parametrize("name", RD.MODEL_NAMES)
def test_oracle_get_new_rects_matches_the_reference_vectors(name, tmp_path):
    """The oracle's box regression (tracking.cpp:90-166) against the outputs of the
    reference's compiled get_new_rects, kept records and records past the borders."""
    boxes, want = RD.get_new_rects_vectors(name)
    paths = RD.write_model_csv(RD.model_dump(name), str(tmp_path), name)
    for ratio in RD.GNR_RATIOS:
        got = O.get_new_rects(O.Model(*paths, ratio), boxes, 640, 480)
        _same_rects(got, want[ratio], (name, ratio))


@needs_ref
@pytest.mark.parametrize("name", RD.MODEL_NAMES)
def test_reference_get_new_rects_reproduces_its_vectors(name):
    boxes, want = RD.get_new_rects_vectors(name)
    paths = [os.path.join(O.REF_SRC_DIR, f"{name}_{k}.csv") for k in ("comp", "root", "part")]
    for ratio in RD.GNR_RATIOS:
        _same_rects(O.ref_get_new_rects(*paths, ratio, boxes, 640, 480), want[ratio], (name, ratio))
