"""A small PNG writer for the tests (the reference reads its depth and mask
frames as PNG): grey or RGB, 8 or 16 bit, a chosen scanline filter per row
and zlib level, so that every filter and block type of the decoder is
exercised."""
import struct
import zlib

import numpy as np


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter_row(row, prev, bpp, f):
    out = bytearray(len(row))
    for x in range(len(row)):
        a = row[x - bpp] if x >= bpp else 0
        b = prev[x]
        c = prev[x - bpp] if x >= bpp else 0
        pred = (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]
        out[x] = (row[x] - pred) & 0xFF
    return bytes(out)


def encode(img, bit_depth=None, filters=None, level=6):
    """img: uint8 or uint16 array [h, w] or [h, w, 3]; filters: one filter type
    per row (cycled), default all 0..4."""
    img = np.asarray(img)
    if bit_depth is None:
        bit_depth = 16 if img.dtype == np.uint16 else 8
    h, w = img.shape[:2]
    ch = 1 if img.ndim == 2 else img.shape[2]
    ctype = {1: 0, 3: 2, 2: 4, 4: 6}[ch]
    if bit_depth == 16:
        raw = img.astype(">u2").tobytes()
    else:
        raw = img.astype(np.uint8).tobytes()
    stride = w * ch * bit_depth // 8
    bpp = max(1, ch * bit_depth // 8)
    filters = list(filters) if filters is not None else [0, 1, 2, 3, 4]
    data = bytearray()
    prev = bytes(stride)
    for y in range(h):
        row = raw[y * stride:(y + 1) * stride]
        f = filters[y % len(filters)]
        data.append(f)
        data += _filter_row(row, prev, bpp, f)
        prev = row

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, bit_depth, ctype, 0, 0, 0)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(bytes(data), level))
            + chunk(b"IEND", b""))


def write(path, img, **kw):
    with open(path, "wb") as f:
        f.write(encode(img, **kw))
