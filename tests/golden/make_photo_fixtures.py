"""Generate tests/golden/photo_fixtures.npz: small real-photograph fixtures
that travel with the repository, so the GPU photograph tests run where the
reference's test photographs are absent.  TEST INFRASTRUCTURE; run where the
reference tree is present (x86-64):

    python tests/golden/make_photo_fixtures.py

Contents, all from the reference's own files and code:
* ``rgba_<name>``: RGBA8 rows (h, 4w) of each fixture as the reference
  harness loads them (its PNG loader, lodepng, compiled from the reference
  tree; alpha forced to 255 as the harness does).  ``patterns`` (32x32) is a
  whole test photograph; the others are crops of photographs (Kodak suite
  images and the harness's default image parrot_red), the crop rectangle
  recorded beside them.
* ``meta``: JSON with, per fixture, the crop, the SHA-256 of the blocks the
  reference encoder itself (goofy::compressDXT1 / compressETC1) writes for
  it, and the harness's getMsePsnr record of those blocks (the oracle's
  restatement, pinned to the harness's printed rows); and the SHA-256 of the
  files the harness writes for ``patterns`` (a run of the harness built with
  its long test list, ENABLE_LONG_TEST_RUN, whose first image it is).
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import run_harness  # noqa: E402
from oracle.build import TEST_DATA  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "photo_fixtures.npz")
# name: (photograph, x, y, width, height); None = the whole photograph
FIXTURES = {
    "patterns": ("patterns", None),
    "kodim03_crop": ("kodim03", (256, 128, 256, 128)),
    "kodim23_crop": ("kodim23", (320, 192, 192, 128)),
    "parrot_red_crop": ("parrot_red", (240, 320, 256, 160)),
}
HARNESS_SUFFIXES = ("original.tga", "baseline.tga", "simd_goofy_dxt1.dds", "simd_goofy_dxt1_decompressed.tga",
                    "simd_goofy_etc1.ktx", "simd_goofy_etc1_decompressed.tga")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(name):
    err, img, w, h = oracle.ref_png_decode(open(os.path.join(TEST_DATA, name + ".png"), "rb").read())
    assert err == 0, name
    img[:, 3::4] = 255
    return img, w, h


def harness_patterns_files():
    """SHA-256 of the files the harness writes for `patterns`: the harness
    built with its long image list runs `patterns` first; the missing
    photographs after it end the run, so its exit status is not checked."""
    run_dir = os.path.join(run_harness.RUN_DIR, "long")
    os.makedirs(os.path.join(run_dir, "test-results"), exist_ok=True)
    binary = os.path.join(run_dir, "goofy_harness_long")
    src = [os.path.join(run_harness.REFERENCE, "Src", f) for f in ("main.cpp", "decoder.cpp",
                                                                    "goofy_tc_reference.cpp")]
    subprocess.run(["g++", "-O2", "-DNDEBUG", "-DENABLE_LONG_TEST_RUN", "-std=c++17", "-msse4.1", "-o", binary] + src
                   + ["-lpthread"], check=True)
    link = os.path.join(run_dir, "test-data")
    if not os.path.islink(link):
        os.symlink(TEST_DATA, link)
    subprocess.run([binary], cwd=run_dir, timeout=900, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    files = {}
    for suffix in HARNESS_SUFFIXES:
        with open(os.path.join(run_dir, "test-results", "patterns_" + suffix), "rb") as f:
            files["patterns_" + suffix] = hashlib.sha256(f.read()).hexdigest()
    return files


def main():
    oracle.build.build()
    ref = oracle.load_ref()
    assert ref is not None, "the reference library is needed (x86-64 with the reference tree)"
    arrays, meta = {}, {"fixtures": {}}
    for key, (photo, crop) in FIXTURES.items():
        img, w, h = load(photo)
        if crop:
            x, y, w, h = crop
            img = np.ascontiguousarray(img[y:y + h, 4 * x:4 * (x + w)])
        assert w % 16 == 0 and h % 4 == 0
        entry = {"photo": photo, "crop": list(crop) if crop else None, "width": w, "height": h,
                 "rgba_sha256": sha(img)}
        for codec, cname in enumerate(("bc1", "etc1s")):
            out = np.zeros((w // 4) * (h // 4) * 8, np.uint8)
            assert ref.ref_compress(codec, out.ctypes.data, img.ctypes.data, w, h, 4 * w) == 0
            dec, bad = oracle.decode(codec, out, w, h)
            entry[cname] = {"sha256": sha(out), "unsupported_blocks": int(bad),
                            "mse_psnr": oracle.mse_psnr(img, dec, w, h)}
        arrays["rgba_" + key] = img
        meta["fixtures"][key] = entry
    meta["harness_files_patterns"] = harness_patterns_files()
    np.savez_compressed(OUT, meta=np.array(json.dumps(meta, sort_keys=True)), **arrays)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
