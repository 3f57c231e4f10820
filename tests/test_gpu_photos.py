"""Real-image regression on the GPU: every reference test photograph the
harness accepts, loaded by the library's PNG loader, encoded through the
drop-in entry points (host buffers, as the harness calls them) and through
one batch launch, gives the reference's blocks; the GPU quality measurement
gives the harness's getMsePsnr record.  Needs the photographs in a folder
named by GOOFY_TEST_DATA; skipped without them."""
import hashlib
import json
import os

import numpy as np
import pytest

import goofy_gb300 as g

pytestmark = pytest.mark.gpu
DIGESTS = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "photo_digests.json")))
TEST_DATA = os.environ.get("GOOFY_TEST_DATA", "")
needs_photos = pytest.mark.skipif(not TEST_DATA or not os.path.isdir(TEST_DATA),
                                  reason="no photograph folder given (GOOFY_TEST_DATA)")


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _names():
    """The digested photographs present in the folder (all of them in a full run)."""
    names = [n for n in sorted(DIGESTS["photos"]) if os.path.exists(os.path.join(TEST_DATA, n + ".png"))]
    assert names, "no digested photograph in " + TEST_DATA
    return names


def _load(name):
    d = DIGESTS["photos"][name]
    img, w, h = g.read_png(os.path.join(TEST_DATA, name + ".png"))
    assert (w, h) == (d["width"], d["height"]) and _sha(img) == d["rgba_sha256"]
    return d, img, w, h


@needs_photos
def test_photographs_dropin_and_quality(cuda):
    for name in _names():
        d, img, w, h = _load(name)
        d_src = cuda.from_numpy(img.reshape(-1)).cuda()
        for codec, (cname, fn) in enumerate((("bc1", g.compressDXT1), ("etc1s", g.compressETC1))):
            out = np.zeros(g.out_size(w, h), np.uint8)
            assert fn(out, img, w, h, 4 * w) == 0
            assert _sha(out) == d[cname]["sha256"], (name, cname)
            q = g.mse_psnr(codec, cuda.from_numpy(out).cuda(), d_src, w, h, 4 * w)
            assert q["unsupported_blocks"] == 0
            for k, v in d[cname]["mse_psnr"].items():
                # luma: exact integers here, the harness's rounded 0.21 / 0.72 / 0.07 products there
                tol = 1e-10 if k.endswith("_y") else 1e-12
                assert q[k] == pytest.approx(v, rel=tol), (name, cname, k)


@needs_photos
def test_all_photographs_in_one_batch(cuda):
    items = []
    for name in _names():
        d, img, w, h = _load(name)
        src = cuda.from_numpy(img.reshape(-1)).cuda()
        for codec, cname in enumerate(("bc1", "etc1s")):
            items.append((src, cuda.zeros(g.out_size(w, h), dtype=cuda.uint8, device="cuda"), w, h, codec,
                          d[cname]["sha256"]))
    b = g.Batch(len(items))
    try:
        assert b.encode([(s, o, w, h, 4 * w, c) for s, o, w, h, c, _ in items]) == g.OK
        cuda.cuda.synchronize()
    finally:
        b.close()
    for s, o, w, h, c, want in items:
        assert _sha(o.cpu().numpy()) == want


@needs_photos
def test_tool_writes_the_harness_files(cuda, tmp_path):
    """`tool run --out` on parrot_red writes the harness's files byte for byte:
    DDS / KTX, the GPU-decoded TGA images, the original and the baseline."""
    import contextlib
    import io

    from goofy_gb300 import tool

    with contextlib.redirect_stdout(io.StringIO()):
        assert tool.main(["run", "--data", TEST_DATA, "--images", "parrot_red", "--iterations", "2",
                          "--out", str(tmp_path)]) == 0
    got = {p.name.replace(tool.ENCODER, "simd_goofy"): hashlib.sha256(p.read_bytes()).hexdigest()
           for p in tmp_path.iterdir()}
    assert got == DIGESTS["harness_files"]
