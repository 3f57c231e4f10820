"""The oracle's decoder and PSNR (the reference harness's quality check)
pinned against the reference: its own block decoders compiled from
Src/decoder.cpp, and the RGB-PSNR its harness reports on parrot_red
(36.82625 dB BC1, 36.15746 dB ETC1), where the reference tree exists."""
import os

import numpy as np
import pytest

import oracle
from oracle.build import TEST_DATA
from goofy_gb300 import workloads

PARROT = os.path.join(TEST_DATA, "parrot_red.png")


def _ref():
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("reference not available on this host")
    return ref


def _decode_blocks(lib_fn, codec, blocks):
    out = np.zeros((len(blocks), 64), np.uint8)
    for i, b in enumerate(blocks):
        lib_fn(codec, np.ascontiguousarray(b).ctypes.data, out[i].ctypes.data)
    return out


def _random_etc1_blocks(rng, n):
    """ETC1 individual / differential blocks (no ETC2-mode overflow), both flips."""
    blocks = rng.integers(0, 256, (n, 8), dtype=np.uint8)
    for b in blocks:
        if b[3] & 2:  # differential: keep base + delta inside 0..31
            for c in range(3):
                base = int(b[c]) >> 3
                d = int(b[c]) & 7
                d = d - 8 if d >= 4 else d
                if not 0 <= base + d <= 31:
                    b[c] = (base << 3) | (0 if base + d < 0 or base + d > 31 else b[c] & 7)
    return blocks


def test_decoder_matches_reference_decoder(built, golden):
    ref = _ref()
    rng = np.random.default_rng(42)
    bc1 = [golden["kat_bc1"].reshape(-1, 8), rng.integers(0, 256, (4000, 8), dtype=np.uint8)]
    etc = [golden["kat_etc1s"].reshape(-1, 8), _random_etc1_blocks(rng, 4000)]
    for codec, sets in ((0, bc1), (1, etc)):
        for blocks in sets:
            got = _decode_blocks(oracle.load().oracle_decode_block, codec, blocks)
            want = _decode_blocks(ref.ref_decode_block, codec, blocks)
            np.testing.assert_array_equal(got, want)


def test_decode_image_and_error_sums(built):
    img = workloads.scene(64, 32, 9)
    for codec in (0, 1):
        blocks = oracle.encode(codec, img, 64, 32)
        dec, bad = oracle.decode(codec, blocks, 64, 32)
        assert bad == 0
        sums = oracle.sq_error(img, dec, 64, 32)
        d = img.astype(np.int64) - dec.astype(np.int64)
        np.testing.assert_array_equal(sums, [(d[:, c::4] ** 2).sum() for c in range(4)])
        assert sums[3] == 0  # alpha 255 in and out
        assert 25.0 < oracle.psnr_rgb(sums, 64, 32) < 60.0


def test_psnr_matches_reference_harness_on_parrot_red(built):
    """Src/main.cpp's reported RGB-PSNR for the reference encoder on
    parrot_red (736x980): BC1 36.82625 dB, ETC1 36.15746 dB."""
    if not os.path.exists(PARROT):
        pytest.skip("reference test images not available on this host")
    from tests.pngread import read_png_rgba

    img, w, h = read_png_rgba(PARROT)
    assert (w, h) == (736, 980)
    for codec, want in ((0, 36.82625), (1, 36.15746)):
        blocks = oracle.encode(codec, img, w, h, any_width=False)
        dec, bad = oracle.decode(codec, blocks, w, h)
        assert bad == 0
        psnr = oracle.psnr_rgb(oracle.sq_error(img, dec, w, h), w, h)
        assert abs(psnr - want) < 5e-6, (codec, psnr)
