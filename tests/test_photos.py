"""Real-image regression on the reference's own test photographs (CPU side):
the committed digests agree with the harness's printed result rows; where the
photographs are present, the library's PNG loader gives the harness's pixels
and the oracle gives the reference's blocks and quality numbers on every
photograph the harness accepts."""
import hashlib
import json
import os

import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from oracle.build import TEST_DATA

DIGESTS = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "photo_digests.json")))
CODECS = {"DXT1": "bc1", "ETC1": "etc1s"}


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_digests_agree_with_the_harness_output():
    rows = [r for r in DIGESTS["harness_rows"] if r["encoder"] == "simd_goofy"]
    assert {r["format"] for r in rows} == {"DXT1", "ETC1"}
    for r in rows:
        q = DIGESTS["photos"][r["image"]][CODECS[r["format"]]]["mse_psnr"]
        for k in ("mse_r", "mse_g", "mse_b", "mse_max", "mse_rgb", "mse_y", "psnr_r", "psnr_g", "psnr_b", "psnr_min",
                  "psnr_rgb", "psnr_y"):
            assert "%3.5f" % q[k] == r[k], (r["image"], r["format"], k)


def luma_mse(src, dec, w, h):
    """mseY from exact integers (what the GPU measurement sums): the harness's 0.21 R + 0.72 G + 0.07 B (R =
    byte 2 of a little-endian pixel) scaled by 100."""
    d = src.reshape(h, w, 4)[..., :3].astype(np.int64) - dec.reshape(h, w, 4)[..., :3].astype(np.int64)
    y = 21 * d[..., 2] + 72 * d[..., 1] + 7 * d[..., 0]
    return float((y * y).sum()) / 10000.0 / (w * h)


@pytest.mark.skipif(not os.path.isdir(TEST_DATA), reason="reference test photographs not present")
@pytest.mark.parametrize("name", sorted(DIGESTS["photos"]))
def test_photograph_against_reference_digest(built, name):
    d = DIGESTS["photos"][name]
    img, w, h = g.read_png(os.path.join(TEST_DATA, name + ".png"))
    assert (w, h) == (d["width"], d["height"])
    assert _sha(img) == d["rgba_sha256"]
    for codec, cname in enumerate(("bc1", "etc1s")):
        out = oracle.encode(codec, img, w, h, any_width=False)
        assert _sha(out) == d[cname]["sha256"]
        dec, bad = oracle.decode(codec, out, w, h)
        assert bad == d[cname]["unsupported_blocks"] == 0
        q = oracle.mse_psnr(img, dec, w, h)
        for k, v in d[cname]["mse_psnr"].items():
            assert q[k] == pytest.approx(v, rel=1e-12), k
        # exact integers vs the harness's rounded 0.21 / 0.72 / 0.07 products
        assert luma_mse(img, dec, w, h) == pytest.approx(q["mse_y"], rel=1e-10)


HARNESS_FIELDS = ("image", "encoder", "format", "pixels", "time_us", "mps", "mse_r", "mse_g", "mse_b", "mse_max",
                  "mse_rgb", "mse_y", "psnr_r", "psnr_g", "psnr_b", "psnr_min", "psnr_rgb", "psnr_y", "delta_min",
                  "delta_rgb", "delta_y")


@pytest.mark.skipif(not os.path.isdir(TEST_DATA), reason="reference test photographs not present")
def test_tool_rows_match_the_harness_rows(built):
    """The command-line tool's result rows (its RGB565 baseline, quality
    record and formatting) equal the harness's printed rows field for field,
    timings aside; the Goofy rows take the quality record of the reference's
    blocks from the digests, which the GPU measurement must reproduce."""
    from goofy_gb300 import tool

    rows = {(r["encoder"], r["format"]): r for r in DIGESTS["harness_rows"]}
    base_row = rows[("Baseline (Downsample x2)", "RGB565")]
    name = base_row["image"]
    img, w, h = g.read_png(os.path.join(TEST_DATA, name + ".png"))
    base = tool.mse_psnr_images(img, tool.baseline_rgb565(img, w, h), w, h)
    got = dict(zip(HARNESS_FIELDS, tool.result_row(name, "Baseline (Downsample x2)", "RGB565", w * h, 0, base,
                                                   base).split(";")))
    assert got == base_row
    for fmt, cname in (("ETC1", "etc1s"), ("DXT1", "bc1")):
        want = rows[("simd_goofy", fmt)]
        q = DIGESTS["photos"][name][cname]["mse_psnr"]
        got = dict(zip(HARNESS_FIELDS, tool.result_row(name, "simd_goofy", fmt, w * h, float(want["time_us"]), q,
                                                       base).split(";")))
        for k in HARNESS_FIELDS:
            if k != "mps":  # the harness divides its rounded-to-print time; mps follows from time_us
                assert got[k] == want[k], (fmt, k)


@pytest.mark.skipif(not os.path.isdir(TEST_DATA), reason="reference test photographs not present")
def test_harness_files_byte_for_byte(built):
    """The files the harness wrote for parrot_red -- DDS, KTX, decoded TGA
    images, the original and the RGB565 baseline -- equal, byte for byte, the
    library's container / TGA writers fed with the oracle's blocks and decode
    and the command-line tool's baseline."""
    from goofy_gb300 import tool

    want = DIGESTS["harness_files"]
    img, w, h = g.read_png(os.path.join(TEST_DATA, "parrot_red.png"))
    got = {"parrot_red_original.tga": g.tga(img, w, h),
           "parrot_red_baseline.tga": g.tga(tool.baseline_rgb565(img, w, h), w, h)}
    for codec, kind, ext in ((0, "dxt1", "dds"), (1, "etc1", "ktx")):
        blocks = oracle.encode(codec, img, w, h, any_width=False)
        dec, _ = oracle.decode(codec, blocks, w, h)
        got["parrot_red_simd_goofy_%s.%s" % (kind, ext)] = g.container(codec, [(blocks, w, h)])
        got["parrot_red_simd_goofy_%s_decompressed.tga" % kind] = g.tga(dec, w, h)
    assert {k: hashlib.sha256(v).hexdigest() for k, v in got.items()} == want


def test_photo_fixtures_match_the_oracle(built):
    """The committed photograph fixtures (tests/golden/photo_fixtures.npz, the
    GPU photograph tests' inputs where the photographs are absent): the whole
    photograph is the digested one, and the oracle gives the recorded
    reference blocks and quality record of every fixture."""
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "photo_fixtures.npz"))
    meta = json.loads(str(d["meta"]))
    assert set(meta["fixtures"]) >= {"patterns", "kodim03_crop", "kodim23_crop", "parrot_red_crop"}
    assert meta["fixtures"]["patterns"]["rgba_sha256"] == DIGESTS["photos"]["patterns"]["rgba_sha256"]
    for codec in ("bc1", "etc1s"):
        assert meta["fixtures"]["patterns"][codec]["sha256"] == DIGESTS["photos"]["patterns"][codec]["sha256"]
    assert len(meta["harness_files_patterns"]) == 6
    for name, f in meta["fixtures"].items():
        img, w, h = d["rgba_" + name], f["width"], f["height"]
        assert img.shape == (h, 4 * w) and _sha(img) == f["rgba_sha256"]
        for codec, cname in enumerate(("bc1", "etc1s")):
            out = oracle.encode(codec, img, w, h, any_width=False)
            assert _sha(out) == f[cname]["sha256"], (name, cname)
            dec, bad = oracle.decode(codec, out, w, h)
            q = oracle.mse_psnr(img, dec, w, h)
            for k, v in f[cname]["mse_psnr"].items():
                assert q[k] == pytest.approx(v, rel=1e-12), (name, cname, k)
