"""Minimal PNG reader (8-bit RGBA / RGB / gray, non-interlaced) for the goldens."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def read_png(path: str) -> np.ndarray:
    """Returns straight-alpha RGBA uint8 of shape (h, w, 4)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", path
    i, idat, w = 8, b"", None
    while i < len(data):
        n, = struct.unpack(">I", data[i:i + 4])
        t = data[i + 4:i + 8]
        body = data[i + 8:i + 8 + n]
        if t == b"IHDR":
            w, h, bd, ct, _cm, _fm, il = struct.unpack(">IIBBBBB", body)
            assert bd == 8 and il == 0, (path, bd, il)
        elif t == b"IDAT":
            idat += body
        i += 12 + n
    ch = {6: 4, 2: 3, 0: 1, 4: 2}[ct]
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int64)
    pos = 0
    for y in range(h):
        f = raw[pos]
        line = np.frombuffer(raw[pos + 1:pos + 1 + stride], dtype=np.uint8).astype(np.int64)
        pos += 1 + stride
        cur = np.zeros(stride, dtype=np.int64)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                b = prev[x]
                c = prev[x - ch] if x >= ch else 0
                if f == 1:
                    cur[x] = (line[x] + a) & 255
                elif f == 3:
                    cur[x] = (line[x] + ((a + b) >> 1)) & 255
                else:
                    cur[x] = (line[x] + _paeth(a, b, c)) & 255
        out[y] = cur
        prev = cur
    img = out.reshape(h, w, ch)
    if ch == 4:
        return img
    rgba = np.zeros((h, w, 4), np.uint8)
    if ch == 3:
        rgba[..., :3] = img
        rgba[..., 3] = 255
    elif ch == 1:
        rgba[..., :3] = img
        rgba[..., 3] = 255
    else:
        rgba[..., :3] = img[..., :1]
        rgba[..., 3] = img[..., 1]
    return rgba
