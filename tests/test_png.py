"""PNG ingest (goofy_gpu_png_*, the library's replacement for the harness's
loadPngAsRgba8): every colour type, bit depth, filter, interlace method and
DEFLATE block type decodes to the RGBA8 the harness's own loader (lodepng,
compiled from the reference tree where it exists) produces; malformed files
are rejected; the reference's test photographs decode identically."""
import glob
import os
import zlib

import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from oracle.build import TEST_DATA
from tests.pngwrite import expected_rgba, write_png

FORMATS = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
           (4, 8), (4, 16), (6, 8), (6, 16)]
STRATEGIES = [(0, zlib.Z_DEFAULT_STRATEGY), (9, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_FIXED),
              (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE)]


def _case(ctype, depth, w, h, seed, with_trns):
    rng = np.random.default_rng(seed)
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    top = (1 << depth) - 1
    # smooth ramps plus noise, so filters and back-references both get used
    ramp = (np.arange(w)[None, :, None] * 7 + np.arange(h)[:, None, None] * 3) % (top + 1)
    samples = np.where(rng.random((h, w, ch)) < 0.3, rng.integers(0, top + 1, (h, w, ch)), ramp).astype(np.int64)
    palette = trns = None
    if ctype == 3:
        n = min(top + 1, 200)
        palette = rng.integers(0, 256, (n, 3))
        samples[0, 0, 0] = min(top, 250)  # an index past a short palette decodes as opaque black
        if with_trns:
            trns = list(rng.integers(0, 256, n // 2))
    elif with_trns and ctype in (0, 2):
        key = samples[h // 2, w // 2]
        trns = [b for v in key for b in (int(v) >> 8, int(v) & 255)]
    return samples, palette, trns


def _decode(data, opaque=False):
    img, w, h = g.read_png(data, opaque=opaque)
    return img, w, h


@pytest.mark.parametrize("ctype,depth", FORMATS)
@pytest.mark.parametrize("interlace", [0, 1])
def test_formats_decode_like_the_loader(built, ctype, depth, interlace):
    ref = oracle.load_ref()
    for k, (w, h) in enumerate([(1, 1), (3, 7), (37, 23), (64, 9)]):
        samples, palette, trns = _case(ctype, depth, w, h, 10 * depth + ctype + k, with_trns=k % 2 == 1)
        level, strategy = STRATEGIES[k % len(STRATEGIES)]
        data = write_png(samples, ctype, depth, interlace, palette, trns, level=level, strategy=strategy,
                         idat_split=1 + k)
        img, gw, gh = _decode(data)
        assert (gw, gh) == (w, h)
        want = expected_rgba(samples, ctype, depth, palette, trns)
        np.testing.assert_array_equal(img, want)
        if ref is not None:
            err, ref_img, rw, rh = oracle.ref_png_decode(data)
            assert err == 0 and (rw, rh) == (w, h)
            np.testing.assert_array_equal(img, ref_img)
        opaque, _, _ = _decode(data, opaque=True)
        want[:, 3::4] = 255
        np.testing.assert_array_equal(opaque, want)


@pytest.mark.parametrize("level,strategy", STRATEGIES)
def test_every_deflate_block_type(built, level, strategy):
    samples, _, _ = _case(6, 8, 300, 200, 5, False)
    for filters in ((0,), (1,), (2,), (3,), (4,), (0, 1, 2, 3, 4)):
        data = write_png(samples, 6, 8, 0, filters=filters, level=level, strategy=strategy, idat_split=3)
        img, _, _ = _decode(data)
        np.testing.assert_array_equal(img, expected_rgba(samples, 6, 8))


def test_stride_and_buffer_checks(built):
    samples, _, _ = _case(2, 8, 20, 10, 1, False)
    data = write_png(samples, 2, 8)
    img, w, h = g.read_png(data, stride=96)
    np.testing.assert_array_equal(img[:, :80], expected_rgba(samples, 2, 8))
    assert not img[:, 80:].any()
    lib = g.lib()
    buf = np.zeros(10 * 80, np.uint8)
    w, h = g._U32(), g._U32()
    assert lib.goofy_gpu_png_decode(data, len(data), buf.ctypes.data, buf.nbytes - 1, 80, 1, w, h) == g.ERR_TOO_LARGE
    assert (w.value, h.value) == (20, 10)
    assert lib.goofy_gpu_png_decode(data, len(data), buf.ctypes.data, buf.nbytes, 76, 1, w, h) == g.ERR_INVALID
    assert lib.goofy_gpu_png_info(data, len(data), w, h) == g.OK and (w.value, h.value) == (20, 10)


def _corrupt(data, pos, xor=0x01):
    b = bytearray(data)
    b[pos] ^= xor
    return bytes(b)


def test_malformed_files_are_rejected(built):
    samples, _, _ = _case(2, 8, 33, 17, 2, False)
    good = write_png(samples, 2, 8)
    idat = good.index(b"IDAT")
    n = int.from_bytes(good[idat - 4:idat], "big")
    bad = {
        "signature": _corrupt(good, 1),
        "ihdr crc": _corrupt(good, 20),
        "idat crc": _corrupt(good, idat + 4 + n),
        "truncated": good[:idat + n // 2],
        "no iend": good[:-12],
        "empty": b"",
    }
    # payload damage with CRCs fixed up: bad Adler-32, bad filter byte
    import struct

    def refit(payload):
        body = b"IDAT" + payload
        return good[:idat - 4] + struct.pack(">I", len(payload)) + body + \
            struct.pack(">I", zlib.crc32(body) & 0xFFFFFFFF) + good[idat + 4 + n + 4:]

    z = good[idat + 4:idat + 4 + n]
    bad["adler"] = refit(z[:-1] + bytes([z[-1] ^ 1]))
    raw = bytearray(zlib.decompress(z))
    raw[0] = 7
    bad["filter type"] = refit(zlib.compress(bytes(raw)))
    bad["short data"] = refit(zlib.compress(bytes(raw[:-5])))
    for name, data in bad.items():
        with pytest.raises(ValueError):
            _decode(data)
        if oracle.load_ref() is not None and data:
            assert oracle.ref_png_decode(data)[0] != 0, name  # the loader rejects it too


@pytest.mark.skipif(not os.path.isdir(TEST_DATA), reason="reference test photographs not present")
def test_reference_photographs_decode_like_the_loader(built):
    files = sorted(glob.glob(os.path.join(TEST_DATA, "*.png")))
    assert files
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("reference loader not built here")
    for f in files:
        data = open(f, "rb").read()
        img, w, h = _decode(data)
        err, want, rw, rh = oracle.ref_png_decode(data)
        assert err == 0 and (w, h) == (rw, rh), f
        np.testing.assert_array_equal(img, want, err_msg=f)


def test_damaged_files_never_crash(built):
    """Random byte flips, truncations and chunk-length edits of valid files:
    the decoder returns a decoded image or an error, never reads or writes
    out of bounds (this test would crash the process), and with the CRCs
    intact agrees with the loader (lodepng) on whether the file decodes and
    on the pixels when it does."""
    rng = np.random.default_rng(99)
    seeds = []
    for ctype, depth in ((2, 8), (6, 8), (3, 4), (0, 16), (4, 8)):
        samples, palette, trns = _case(ctype, depth, 23, 19, ctype * 7 + depth, False)
        for interlace in (0, 1):
            seeds.append(write_png(samples, ctype, depth, interlace, palette, trns, idat_split=2))
    for k in range(400):
        data = bytearray(seeds[k % len(seeds)])
        kind = k % 4
        if kind == 0:  # flip a few payload bytes
            for _ in range(int(rng.integers(1, 4))):
                data[int(rng.integers(8, len(data)))] ^= int(rng.integers(1, 256))
        elif kind == 1:  # truncate
            data = data[:int(rng.integers(8, len(data)))]
        elif kind == 2:  # corrupt a chunk length
            pos = 8 + 4 * int(rng.integers(0, 4))
            data[pos:pos + 4] = int(rng.integers(0, 2 ** 32)).to_bytes(4, "big")
        else:  # damage the compressed data and fix the CRC, so only inflate can catch it
            idat = data.find(b"IDAT")
            n = int.from_bytes(data[idat - 4:idat], "big")
            data[idat + 4 + int(rng.integers(0, n))] ^= int(rng.integers(1, 256))
            crc = zlib.crc32(bytes(data[idat:idat + 4 + n])) & 0xFFFFFFFF
            data[idat + 4 + n:idat + 8 + n] = crc.to_bytes(4, "big")
        try:
            img, w, h = g.read_png(bytes(data), opaque=False)
            ok = True
        except ValueError:
            ok = False
        if kind == 3 and oracle.load_ref() is not None:
            err, want, _, _ = oracle.ref_png_decode(bytes(data))
            assert ok == (err == 0), (k, err)
            if ok:
                np.testing.assert_array_equal(img, want)
