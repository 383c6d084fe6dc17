"""Tiny PNG decoder for the tests (8-bit, filter 0 as written by the
library, plus the standard filters for robustness)."""
import struct
import zlib

import numpy as np


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(typ + body) & 0xffffffff == crc
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            ch = {0: 1, 2: 3, 6: 4}[ctype]
            assert depth == 8
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        row = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        if f == 0:
            cur = row
        elif f == 2:
            cur = (row + prev) & 255
        else:
            cur = row.copy()
            for i in range(stride):
                left = cur[i - ch] if i >= ch else 0
                up = prev[i]
                if f == 1:
                    cur[i] = (row[i] + left) & 255
                elif f == 3:
                    cur[i] = (row[i] + (left + up) // 2) & 255
                else:
                    ul = prev[i - ch] if i >= ch else 0
                    p = left + up - ul
                    pa, pb, pc = abs(p - left), abs(p - up), abs(p - ul)
                    pr = left if pa <= pb and pa <= pc else (up if pb <= pc else ul)
                    cur[i] = (row[i] + pr) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, ch) if ch > 1 else out.reshape(h, w)
