"""PNG writer for the ingest tests (test utility): any colour type / bit
depth, Adam7 or plain, a chosen scanline filter per row, a chosen zlib
strategy and IDAT chunking, so every branch of a decoder gets bytes to read."""
import struct
import zlib

import numpy as np

CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _pack_rows(samples, depth):
    """(h, w, ch) integer samples -> (h, rowbytes) bytes, big-endian / MSB-first."""
    h, w, ch = samples.shape
    if depth == 16:
        s = samples.astype(">u2").reshape(h, w * ch)
        return s.view(np.uint8).reshape(h, 2 * w * ch)
    if depth == 8:
        return samples.astype(np.uint8).reshape(h, w * ch)
    per = 8 // depth
    padded = np.zeros((h, -(-w // per) * per), np.uint16)
    padded[:, :w] = samples[..., 0]
    g = padded.reshape(h, -1, per)
    out = np.zeros(g.shape[:2], np.uint16)
    for k in range(per):
        out |= g[..., k] << (8 - depth * (k + 1))
    return out.astype(np.uint8)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter(rows, bpp, kinds):
    out = []
    prev = np.zeros(rows.shape[1], np.int32)
    for y, row in enumerate(rows.astype(np.int32)):
        f = kinds[y % len(kinds)]
        a = np.concatenate([np.zeros(bpp, np.int32), row[:-bpp]]) if len(row) > bpp else np.zeros_like(row)
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]]) if len(row) > bpp else np.zeros_like(row)
        pred = [0, a, prev, (a + prev) >> 1, _paeth(a, prev, c)][f]
        out.append(bytes([f]) + ((row - pred) & 0xFF).astype(np.uint8).tobytes())
        prev = row
    return b"".join(out)


def write_png(samples, ctype, depth, interlace=0, palette=None, trns=None, filters=(0, 1, 2, 3, 4),
              level=6, strategy=zlib.Z_DEFAULT_STRATEGY, idat_split=1):
    """`samples`: (h, w, channels) integers of the colour type's channel count."""
    h, w, ch = samples.shape
    assert ch == CHANNELS[ctype]
    bpp = max(1, depth * ch // 8)
    raw = []
    for (x0, y0, dx, dy) in (ADAM7 if interlace else ((0, 0, 1, 1),)):
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] and sub.shape[1]:
            raw.append(_filter(_pack_rows(sub, depth), bpp, filters))
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    data = co.compress(b"".join(raw)) + co.flush()
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    out += _chunk(b"tEXt", b"Comment\x00ancillary chunks are skipped")
    if palette is not None:
        out += _chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        out += _chunk(b"tRNS", bytes(trns))
    step = -(-len(data) // idat_split)
    for i in range(0, len(data), step):
        out += _chunk(b"IDAT", data[i:i + step])
    return out + _chunk(b"IEND", b"")


def expected_rgba(samples, ctype, depth, palette=None, trns=None):
    """8-bit RGBA by the loader's conversion rules: 16-bit keeps the high
    byte, low-depth grey scales by 255/(2^depth-1), palette indices past the
    palette give opaque black, tRNS makes the key colour transparent."""
    h, w, _ = samples.shape
    s = samples.astype(np.int64)
    out = np.zeros((h, w, 4), np.uint8)
    out[..., 3] = 255
    hi = (lambda v: v >> 8) if depth == 16 else (lambda v: v)
    if ctype == 0:
        g = s[..., 0] * 255 // ((1 << depth) - 1) if depth < 8 else hi(s[..., 0])
        out[..., :3] = g[..., None]
        if trns is not None:
            key = trns[0] << 8 | trns[1]
            out[..., 3] = np.where(s[..., 0] == key, 0, 255)
    elif ctype == 2:
        out[..., :3] = hi(s)
        if trns is not None:
            key = [trns[2 * c] << 8 | trns[2 * c + 1] for c in range(3)]
            out[..., 3] = np.where((s[..., 0] == key[0]) & (s[..., 1] == key[1]) & (s[..., 2] == key[2]), 0, 255)
    elif ctype == 3:
        pal = np.zeros((256, 4), np.uint8)
        pal[:, 3] = 255
        n = len(palette)
        pal[:n, :3] = palette
        if trns is not None:
            pal[:len(trns), 3] = trns
        out[:] = pal[s[..., 0]]
    elif ctype == 4:
        out[..., :3] = hi(s[..., :1])
        out[..., 3] = hi(s[..., 1])
    else:
        out[:] = hi(s)
    return out.reshape(h, 4 * w)
