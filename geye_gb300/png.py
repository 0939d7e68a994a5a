"""PNG reader for 8-bit, non-interlaced images, in numpy and zlib only.

The reference reads its test frames with OpenCV's image loader
(CAR_TRACKING/showboxes.cpp:548 `load_suc_image`, frames named by
CAR_TRACKING/MODEL_info.h:51), which hands the detector an IplImage of
interleaved B,G,R bytes.  OpenCV is not part of this library, so this module
decodes the frames itself: the chunk stream with CRC checks, zlib inflate of
the IDAT data, and the five row filters of the PNG specification (None, Sub,
Up, Average, Paeth; ISO/IEC 15948 section 9).  `load_bgr` returns the same
height x width x 3 B,G,R array the reference's IplImage holds.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 4: 2, 6: 4}   # colour type -> samples per pixel (8-bit only)


class PngError(ValueError):
    pass


def _chunks(data: bytes):
    if data[:8] != _SIG:
        raise PngError("not a PNG file (bad signature)")
    pos = 8
    while pos + 12 <= len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        if len(body) != n or zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise PngError(f"chunk {kind!r} at byte {pos} is truncated or fails its CRC")
        yield kind, body
        pos += 12 + n
        if kind == b"IEND":
            return
    raise PngError("no IEND chunk")


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    """Undoes the per-row filters; returns h x stride bytes."""
    if len(raw) != h * (stride + 1):
        raise PngError(f"inflated data has {len(raw)} bytes, expected {h * (stride + 1)}")
    rows = np.frombuffer(raw, np.uint8).reshape(h, stride + 1)
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.uint8)
    for y in range(h):
        ft = int(rows[y, 0])
        cur = rows[y, 1:]
        if ft == 0:
            line = cur.copy()
        elif ft == 1:        # Sub: x + a, a running sum per sample position mod 256
            line = np.cumsum(cur.reshape(-1, bpp), axis=0, dtype=np.uint8).reshape(-1)
        elif ft == 2:        # Up: x + b
            line = (cur.astype(np.uint16) + prev).astype(np.uint8)
        elif ft == 3:        # Average: x + floor((a + b) / 2), sequential in a
            line = _avg_slow(cur, prev, bpp)
        elif ft == 4:        # Paeth: x + predictor(a, b, c), sequential in a
            line = _paeth_slow(cur, prev, bpp)
        else:
            raise PngError(f"row {y}: unknown filter type {ft}")
        out[y] = line
        prev = line
    return out


def _avg_slow(cur, prev, bpp):
    b = bytearray(cur.tobytes())
    p = prev.tobytes()
    for i in range(len(b)):
        a = b[i - bpp] if i >= bpp else 0
        b[i] = (b[i] + ((a + p[i]) >> 1)) & 0xFF
    return np.frombuffer(bytes(b), np.uint8)


def _paeth_slow(cur, prev, bpp):
    b = bytearray(cur.tobytes())
    p = prev.tobytes()
    for i in range(len(b)):
        a = b[i - bpp] if i >= bpp else 0
        up = p[i]
        c = p[i - bpp] if i >= bpp else 0
        est = a + up - c
        pa, pb, pc = abs(est - a), abs(est - up), abs(est - c)
        pred = a if (pa <= pb and pa <= pc) else (up if pb <= pc else c)
        b[i] = (b[i] + pred) & 0xFF
    return np.frombuffer(bytes(b), np.uint8)


def decode(data: bytes) -> np.ndarray:
    """PNG bytes -> height x width x channels uint8 array in the file's sample order."""
    ihdr = None
    idat = []
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
    if ihdr is None:
        raise PngError("no IHDR chunk")
    w, h, depth, ctype, comp, filt, interlace = ihdr
    if depth != 8 or ctype not in _CHANNELS or comp != 0 or filt != 0 or interlace != 0:
        raise PngError(f"unsupported PNG: depth {depth}, colour type {ctype}, interlace {interlace} "
                       "(8-bit non-interlaced grey/RGB/RGBA only)")
    ch = _CHANNELS[ctype]
    try:
        raw = zlib.decompress(b"".join(idat))
    except zlib.error as e:
        raise PngError(f"IDAT stream does not inflate: {e}") from e
    return _unfilter(raw, h, w * ch, ch).reshape(h, w, ch)


def load_bgr(path: str) -> np.ndarray:
    """Reads a PNG as the reference's IplImage holds it: height x width x 3, B,G,R, uint8."""
    with open(path, "rb") as f:
        img = decode(f.read())
    ch = img.shape[2]
    if ch == 1 or ch == 2:
        img = np.repeat(img[:, :, :1], 3, axis=2)
    return np.ascontiguousarray(img[:, :, 2::-1] if ch >= 3 else img)
