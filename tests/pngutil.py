"""PNG writer/reader for tests (numpy + zlib): writes real deflate streams (fixed and dynamic Huffman blocks)
with every row filter, so the library's own decoder is exercised on what image tools produce."""
import struct
import zlib

import numpy as np


def _chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def write_png(path, img, level=6):
    """img: h x w u8 (gray) or h x w x 3 u8 in R, G, B order (as stored in PNG). Row k uses filter k % 5."""
    a = np.asarray(img, np.uint8)
    ctype, bpp = (0, 1) if a.ndim == 2 else (2, 3)
    h, w = a.shape[:2]
    rows = a.reshape(h, -1).astype(np.int64)
    out = bytearray()
    prev = np.zeros(w * bpp, np.int64)
    for y in range(h):
        cur = rows[y]
        left = np.concatenate([np.zeros(bpp, np.int64), cur[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int64), prev[:-bpp]])
        ft = y % 5
        pred = [0 * cur, left, prev, (left + prev) // 2, _paeth(left, prev, upleft)][ft]
        out.append(ft)
        out += ((cur - pred) % 256).astype(np.uint8).tobytes()
        prev = cur
    ihdr = struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(bytes(out), level)) + \
        _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(data)


def read_png_gray(path):
    """Reads the gray 8- or 16-bit, filter-0 PNGs the CLI writes."""
    with open(path, "rb") as f:
        data = f.read()
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        t = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if t == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
        elif t == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    bps = depth // 8
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + w * bps)
    assert (rows[:, 0] == 0).all()
    px = rows[:, 1:]
    if depth == 16:
        return (px[:, 0::2].astype(np.uint16) << 8) | px[:, 1::2]
    return px.copy()
