"""Generate tests/golden/goofy_golden.npz from the REFERENCE encoder itself.

Runs goofy::compressDXT1 / goofy::compressETC1 compiled from the reference's
own header (oracle/_ref/libgoofy_ref.so, built by oracle/build.py where the
reference tree exists) on:

* ``kat``   -- 2048 hand-built blocks (64 x 128 px): constant blocks at the
               byte extremes, two-colour blocks, a grey ramp giving every
               luma range 0..255 (so every ETC1 control-byte run and both
               edges of each run), low-contrast noise around random colours,
               i.i.d. noise, the 5-bit quantiser edges 0/1/7/8/9/15/16/17/
               247/248/255, and random alpha on top of all of it;
* ``cfg0``  -- the 256x256 scene, seed 0 (input pinned by its SHA-256);
* ``stress``-- the four degenerate quarters at 256x256, seed 2.

The inputs of ``kat`` are stored; ``cfg0`` / ``stress`` are regenerated by
goofy_gb300.workloads on any host and checked against the stored hash.
Run:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "goofy_golden.npz")


def kat_image():
    rng = np.random.default_rng(20240601)
    blocks = []

    def add(b):
        blocks.append(np.asarray(b, np.uint8).reshape(4, 4, 4))

    for v in (0, 1, 7, 8, 9, 15, 16, 17, 127, 128, 247, 248, 254, 255):
        add(np.full((4, 4, 4), v))
    for r in range(256):  # grey ramp: min 0, max r -> luma range r
        b = np.zeros((4, 4, 4), np.int64)
        vals = np.linspace(0, r, 16).round().astype(np.int64)
        b[..., :3] = rng.permutation(vals).reshape(4, 4, 1)
        b[..., 3] = 255
        add(b)
    for lo in (0, 30, 100, 200):  # ranges offset from zero
        for r in range(0, 256 - lo, 3):
            b = np.zeros((4, 4, 4), np.int64)
            b[..., :3] = rng.integers(lo, lo + r + 1, (4, 4, 1))
            b.reshape(16, 4)[0, :3] = lo
            b.reshape(16, 4)[1, :3] = lo + r
            b[..., 3] = 255
            add(b)
    edges = np.array([0, 1, 7, 8, 9, 15, 16, 17, 247, 248, 255])
    while len(blocks) < 1024:
        kind = len(blocks) % 4
        if kind == 0:  # two colours
            c = rng.integers(0, 256, (2, 4))
            add(c[rng.integers(0, 2, 16)])
        elif kind == 1:  # low contrast
            base = rng.integers(0, 256, 4)
            add(np.clip(base + rng.integers(-12, 13, (16, 4)), 0, 255))
        elif kind == 2:
            add(rng.integers(0, 256, (16, 4)))
        else:
            add(edges[rng.integers(0, len(edges), (16, 4))])
    while len(blocks) < 2048:  # random mixes with independent channel spreads
        spread = rng.integers(0, 256, 3)
        base = rng.integers(0, 256, 3)
        b = np.zeros((16, 4), np.int64)
        for c in range(3):
            b[:, c] = np.clip(base[c] + rng.integers(-spread[c], spread[c] + 1, 16), 0, 255)
        b[:, 3] = rng.integers(0, 256, 16)
        add(b)
    arr = np.stack(blocks)  # (2048, 4, 4, 4)
    arr[:, :, :, 3] = rng.integers(0, 256, arr.shape[:3])  # alpha must not matter
    # tile as 32 block rows x 64 blocks -> 256 x 128 pixels
    grid = arr.reshape(32, 64, 4, 4, 4).transpose(0, 2, 1, 3, 4).reshape(128, 256 * 4)
    return np.ascontiguousarray(grid), 256, 128


def main():
    from oracle import build as oracle_build
    from oracle import load_ref
    from goofy_gb300 import build as lib_build
    from goofy_gb300 import workloads

    oracle_build.build()
    lib_build.build()
    ref = load_ref()
    if ref is None:
        raise SystemExit("the reference encoder is not available on this host")

    def run(codec, img, w, h):
        buf = np.empty(img.size + 64, np.uint8)
        off = (-buf.ctypes.data) % 64  # the reference loads aligned 16-byte vectors
        a = buf[off:off + img.size].reshape(img.shape)
        a[...] = img
        out = np.zeros((w // 4) * (h // 4) * 8, np.uint8)
        assert ref.ref_compress(codec, out.ctypes.data, a.ctypes.data, w, h, img.strides[0]) == 0
        return out

    kat, kw, kh = kat_image()
    cfg0 = workloads.scene(256, 256, 0)
    stress = workloads.stress(256, 256, 2)
    data = {
        "kat_input": kat, "kat_width": kw, "kat_height": kh,
        "kat_bc1": run(0, kat, kw, kh), "kat_etc1s": run(1, kat, kw, kh),
        "cfg0_sha256": hashlib.sha256(np.ascontiguousarray(cfg0).tobytes()).hexdigest(),
        "cfg0_bc1": run(0, cfg0, 256, 256), "cfg0_etc1s": run(1, cfg0, 256, 256),
        "stress_sha256": hashlib.sha256(np.ascontiguousarray(stress).tobytes()).hexdigest(),
        "stress_bc1": run(0, stress, 256, 256), "stress_etc1s": run(1, stress, 256, 256),
    }
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
