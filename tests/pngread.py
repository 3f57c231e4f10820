"""Minimal PNG reader for the real-image checks (test utility): 8-bit
greyscale / RGB / RGBA / palette, non-interlaced, all five scanline filters.
Returns RGBA8 with alpha forced to 255, as the reference harness loads its
test images (Src/main.cpp:318-338)."""
import struct
import zlib

import numpy as np


def _paeth_row(raw, prior, bpp):
    out = raw.astype(np.int32)
    prior = prior.astype(np.int32)
    for i in range(len(out)):
        a = out[i - bpp] if i >= bpp else 0
        b = prior[i]
        c = prior[i - bpp] if i >= bpp else 0
        p = a + b - c
        pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
        pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
        out[i] = (out[i] + pred) & 0xFF
    return out.astype(np.uint8)


def read_png_rgba(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos, idat, plte = 8, [], None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    assert depth == 8 and interlace == 0, "only 8-bit non-interlaced PNGs"
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = channels
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(h, 1 + w * bpp)
    rows = np.zeros((h, w * bpp), np.uint8)
    prior = np.zeros(w * bpp, np.uint8)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:]
        if f == 0:
            cur = line.copy()
        elif f == 1:
            cur = line.copy()
            for c in range(bpp):
                cur[c::bpp] = np.cumsum(line[c::bpp].astype(np.uint32)).astype(np.uint8)
        elif f == 2:
            cur = (line.astype(np.uint16) + prior).astype(np.uint8)
        elif f == 3:
            cur = line.astype(np.int32)
            for i in range(len(cur)):
                a = int(cur[i - bpp]) if i >= bpp else 0
                cur[i] = (int(line[i]) + ((a + int(prior[i])) >> 1)) & 0xFF
            cur = cur.astype(np.uint8)
        else:
            cur = _paeth_row(line, prior, bpp)
        rows[y] = cur
        prior = cur
    px = rows.reshape(h, w, bpp)
    if ctype == 3:
        px = plte[px[..., 0]]
    elif ctype in (0, 4):
        px = np.repeat(px[..., :1], 3, axis=2)
    rgba = np.empty((h, w, 4), np.uint8)
    rgba[..., :3] = px[..., :3]
    rgba[..., 3] = 255
    return rgba.reshape(h, 4 * w), w, h
