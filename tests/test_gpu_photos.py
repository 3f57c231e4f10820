"""Real-image regression on the GPU.  Encoded through the drop-in entry
points (host buffers, as the harness calls them) and through one batch
launch, every photograph gives the reference's blocks, and the GPU quality
measurement gives the harness's getMsePsnr record; the command-line tool
writes the harness's files byte for byte.

Inputs: the photographs in the folder named by GOOFY_TEST_DATA (every test
photograph the harness accepts, loaded by the library's PNG loader), or,
without it, the fixtures committed in tests/golden/photo_fixtures.npz (one
whole test photograph and crops of three others, with the reference
encoder's block digests and the harness's files for the whole one, made by
tests/golden/make_photo_fixtures.py)."""
import hashlib
import json
import os

import numpy as np
import pytest

import goofy_gb300 as g

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIGESTS = json.load(open(os.path.join(GOLDEN, "photo_digests.json")))
TEST_DATA = os.environ.get("GOOFY_TEST_DATA", "")
USE_FOLDER = bool(TEST_DATA) and os.path.isdir(TEST_DATA)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _fixtures():
    d = np.load(os.path.join(GOLDEN, "photo_fixtures.npz"))
    return d, json.loads(str(d["meta"]))


def _photos():
    """(name, record, rgba rows, width, height) of every input photograph."""
    if USE_FOLDER:
        names = [n for n in sorted(DIGESTS["photos"]) if os.path.exists(os.path.join(TEST_DATA, n + ".png"))]
        assert names, "no digested photograph in " + TEST_DATA
        for name in names:
            d = DIGESTS["photos"][name]
            img, w, h = g.read_png(os.path.join(TEST_DATA, name + ".png"))
            assert (w, h) == (d["width"], d["height"]) and _sha(img) == d["rgba_sha256"]
            yield name, d, img, w, h
    else:
        arrays, meta = _fixtures()
        for name, d in sorted(meta["fixtures"].items()):
            img = arrays["rgba_" + name]
            assert _sha(img) == d["rgba_sha256"]
            yield name, d, img, d["width"], d["height"]


def test_photographs_dropin_and_quality(cuda):
    n = 0
    for name, d, img, w, h in _photos():
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
        n += 1
    assert n >= 4


def test_all_photographs_in_one_batch(cuda):
    items = []
    for name, d, img, w, h in _photos():
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


def test_tool_writes_the_harness_files(cuda, tmp_path):
    """`tool run --out` writes the harness's files byte for byte: DDS / KTX,
    the GPU-decoded TGA images, the original and the baseline -- for
    parrot_red from the photograph folder, else for the whole fixture
    photograph `patterns` (written to a PNG file here, as the tool reads
    PNG files)."""
    import contextlib
    import io

    from goofy_gb300 import tool

    if USE_FOLDER:
        data, image, want = TEST_DATA, "parrot_red", DIGESTS["harness_files"]
    else:
        from tests.pngwrite import write_png

        arrays, meta = _fixtures()
        data, image, want = str(tmp_path / "data"), "patterns", meta["harness_files_patterns"]
        os.makedirs(data)
        d = meta["fixtures"]["patterns"]
        rgba = arrays["rgba_patterns"].reshape(d["height"], d["width"], 4)
        with open(os.path.join(data, "patterns.png"), "wb") as f:
            f.write(write_png(rgba, 6, 8))
        assert _sha(g.read_png(os.path.join(data, "patterns.png"))[0]) == d["rgba_sha256"]
    out = tmp_path / "out"
    with contextlib.redirect_stdout(io.StringIO()):
        assert tool.main(["run", "--data", data, "--images", image, "--iterations", "2", "--out", str(out)]) == 0
    got = {p.name.replace(tool.ENCODER, "simd_goofy"): hashlib.sha256(p.read_bytes()).hexdigest()
           for p in out.iterdir()}
    assert got == want
