"""The command-line tool end to end on the GPU: PNG -> DDS / KTX with a
GPU-made mip chain equals the oracle's blocks of the host chain, and the
harness-style run prints one well-formed row set per accepted image."""
import io
import contextlib

import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import tool, workloads
from tests.pngwrite import write_png

pytestmark = pytest.mark.gpu


def _png(tmp_path, name, w, h, seed):
    img = workloads.scene(w, h, seed)
    path = tmp_path / (name + ".png")
    path.write_bytes(write_png(img.reshape(h, w, 4)[..., :3], 2, 8))
    rgba = img.copy()
    rgba.reshape(h, w, 4)[..., 3] = 255
    return path, rgba


@pytest.mark.parametrize("codec,ext", [("bc1", "dds"), ("etc1s", "ktx")])
def test_encode_with_mips(cuda, tmp_path, codec, ext):
    w, h = 256, 64
    path, rgba = _png(tmp_path, "tex", w, h, 5)
    out = tmp_path / ("tex." + ext)
    assert tool.main(["encode", str(path), str(out), "--codec", codec, "--mips"]) == 0
    c = 0 if codec == "bc1" else 1
    chain, cur, cw, ch = [(rgba, w, h)], rgba, w, h
    for _ in workloads.mip_chain(w, h)[1:]:
        cur, cw, ch = workloads.downsample(cur, cw, ch)
        chain.append((cur, cw, ch))
    want = g.container(c, [(oracle.encode(c, im, lw, lh), lw, lh) for im, lw, lh in chain])
    assert out.read_bytes() == want


@pytest.mark.parametrize("mips", [False, True])
def test_encode_both_formats_in_one_pass(cuda, tmp_path, mips):
    """--both writes the DDS and the KTX file from one pass per level; each
    equals the single-format file the oracle's blocks make."""
    w, h = 128, 32
    path, rgba = _png(tmp_path, "tex", w, h, 6)
    argv = ["encode", str(path), str(tmp_path / "tex.dds"), "--both"] + (["--mips"] if mips else [])
    assert tool.main(argv) == 0
    chain, cur, cw, ch = [(rgba, w, h)], rgba, w, h
    for _ in (workloads.mip_chain(w, h)[1:] if mips else []):
        cur, cw, ch = workloads.downsample(cur, cw, ch)
        chain.append((cur, cw, ch))
    for c, ext in ((0, "dds"), (1, "ktx")):
        want = g.container(c, [(oracle.encode(c, im, lw, lh), lw, lh) for im, lw, lh in chain])
        assert (tmp_path / ("tex." + ext)).read_bytes() == want


def test_run_prints_harness_rows(cuda, tmp_path):
    _png(tmp_path, "a", 64, 32, 1)
    _png(tmp_path, "b", 40, 32, 2)  # width % 16 != 0: refused as the harness refuses it
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        assert tool.main(["run", "--data", str(tmp_path), "--iterations", "3", "--out", str(tmp_path / "out")]) == 0
    lines = buf.getvalue().strip().split("\n")
    assert lines[0] == tool.HEADER
    rows = [l.split(";") for l in lines[1:]]
    assert [r[:3] for r in rows] == [["a", "Baseline (Downsample x2)", "RGB565"], ["a", tool.ENCODER, "ETC1"],
                                     ["a", tool.ENCODER, "DXT1"]]
    assert all(len(r) == 21 for r in rows)
    assert sorted(p.name for p in (tmp_path / "out").iterdir()) == [
        "a_baseline.tga", "a_gb300_goofy_dxt1.dds", "a_gb300_goofy_dxt1_decompressed.tga", "a_gb300_goofy_etc1.ktx",
        "a_gb300_goofy_etc1_decompressed.tga", "a_original.tga"]


def test_autotune_records_the_tiles(cuda, tmp_path):
    """`tool autotune` tunes on a small scene and writes this GPU model's
    entries (both codecs and the two-codec pass) into the given cache file."""
    import contextlib
    import io

    from goofy_gb300 import tool

    cache = str(tmp_path / "tiles.txt")
    try:
        with contextlib.redirect_stdout(io.StringIO()) as out:
            assert tool.main(["autotune", "--size", "512", "--reps", "1", "--cache", cache]) == 0
        name, sms = g.device_key(0)
        for c in (g.CODEC_BC1, g.CODEC_ETC1S, g.CODEC_BOTH):
            assert g.tile_cache_lookup(cache, name, sms, c) == g.get_tile(c)
        assert cache in out.getvalue()
    finally:
        g.reset_tiles()
        g.set_tile_cache_path(None)
