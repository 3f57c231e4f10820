"""Generate tests/golden/photo_digests.json: what the REFERENCE produces on
its own test photographs, so the real-image checks can run where only the
photographs (and not the reference) are present.

For every PNG in the reference's test-data/ that its harness accepts
(width % 16 == 0, height % 4 == 0, Src/main.cpp:298-308):

* the image as the harness loads it (lodepng RGBA8, alpha forced to 255) --
  size and SHA-256;
* per codec, the SHA-256 of goofy::compressDXT1 / goofy::compressETC1 output
  (the reference compiled from its own header, oracle/_ref/libgoofy_ref.so)
  and the fourteen getMsePsnr values of that output decoded by the
  harness's decoders (the oracle's restatements, themselves pinned to
  Src/decoder.cpp and to the harness run below);
* the harness's own result rows (Goofy and its RGB565 baseline) for its
  default image (parrot_red), from one run of the harness compiled from the
  reference tree (oracle/run_harness.py), as printed (5 decimals), and the
  SHA-256 of the files that run wrote for Goofy (DDS, KTX, the decoded TGA
  images) and of its original and baseline TGA images.

Run:  python tests/golden/make_photo_digests.py
"""
import glob
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import run_harness  # noqa: E402
from oracle.build import TEST_DATA  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "photo_digests.json")
CODECS = ("bc1", "etc1s")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    oracle.build.build()
    ref = oracle.load_ref()
    assert ref is not None, "the reference library is needed (x86-64 with the reference tree)"
    photos = {}
    for path in sorted(glob.glob(os.path.join(TEST_DATA, "*.png"))):
        name = os.path.basename(path)[:-4]
        err, img, w, h = oracle.ref_png_decode(open(path, "rb").read())
        assert err == 0, path
        if w % 16 or h % 4:
            continue  # the harness refuses these (Src/main.cpp:298-308)
        img[:, 3::4] = 255
        entry = {"width": w, "height": h, "rgba_sha256": sha(img)}
        for codec, cname in enumerate(CODECS):
            out = np.zeros((w // 4) * (h // 4) * 8, np.uint8)
            assert ref.ref_compress(codec, out.ctypes.data, img.ctypes.data, w, h, 4 * w) == 0
            dec, bad = oracle.decode(codec, out, w, h)
            entry[cname] = {"sha256": sha(out), "unsupported_blocks": int(bad),
                            "mse_psnr": oracle.mse_psnr(img, dec, w, h)}
        photos[name] = entry
    harness = [r for r in run_harness.run() if r["encoder"] in ("simd_goofy", "Baseline (Downsample x2)")]
    files = {}
    for suffix in ("original.tga", "baseline.tga", "simd_goofy_dxt1.dds", "simd_goofy_dxt1_decompressed.tga",
                   "simd_goofy_etc1.ktx", "simd_goofy_etc1_decompressed.tga"):
        name = "parrot_red_" + suffix
        with open(os.path.join(run_harness.RUN_DIR, "test-results", name), "rb") as f:
            files[name] = hashlib.sha256(f.read()).hexdigest()
    with open(OUT, "w") as f:
        json.dump({"photos": photos, "harness_rows": harness, "harness_files": files}, f, indent=1, sort_keys=True)
    print("wrote", OUT, len(photos), "photos,", len(harness), "harness rows")


if __name__ == "__main__":
    main()
