"""The tile cache (goofy_gpu_tile_cache_*): tuned image-kernel tiles kept in a
text file per GPU model.  Needs no GPU: entries are written and read back
for a named GPU; malformed lines, tiles the kernels cannot run and entries of
other GPU models are ignored; the path comes from the explicit setting, the
environment or the per-user default."""
import os
import subprocess
import sys

import pytest

import goofy_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GB300 = ("NVIDIA GB300", 152)


@pytest.fixture
def cache(tmp_path, built):
    path = str(tmp_path / "sub" / "tiles.txt")  # the parent folder does not exist yet
    yield path
    g.set_tile_cache_path(None)


def test_round_trip_per_codec_and_gpu(cache):
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_BC1) is None  # no file yet
    assert g.tile_cache_store(cache, *GB300, g.CODEC_BC1, (512, 2, 2), 45.1) == g.OK
    assert g.tile_cache_store(cache, *GB300, g.CODEC_ETC1S, (256, 1, 2), 46.0) == g.OK
    assert g.tile_cache_store(cache, *GB300, g.CODEC_BOTH, (512, 2, 2), 53.3) == g.OK
    assert g.tile_cache_store(cache, "NVIDIA B200", 148, g.CODEC_BC1, (128, 1, 0), 40.0) == g.OK
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_BC1) == (512, 2, 2)
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_ETC1S) == (256, 1, 2)
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_BOTH) == (512, 2, 2)
    assert g.tile_cache_lookup(cache, "NVIDIA B200", 148, g.CODEC_BC1) == (128, 1, 0)
    assert g.tile_cache_lookup(cache, "NVIDIA B200", 148, g.CODEC_ETC1S) is None
    # a foreign GPU: another name, or the same name with another SM count
    assert g.tile_cache_lookup(cache, "NVIDIA GB200", 152, g.CODEC_BC1) is None
    assert g.tile_cache_lookup(cache, "NVIDIA GB300", 148, g.CODEC_BC1) is None
    # a new measurement replaces the entry instead of adding a second one
    assert g.tile_cache_store(cache, *GB300, g.CODEC_BC1, (128, 1, 0), 43.0) == g.OK
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_BC1) == (128, 1, 0)
    lines = [l for l in open(cache).read().splitlines() if not l.startswith("#")]
    assert len(lines) == 4 and sum("|bc1|" in l and "GB300" in l for l in lines) == 1


def test_malformed_and_invalid_lines_are_ignored(cache):
    os.makedirs(os.path.dirname(cache))
    with open(cache, "w") as f:
        f.write("\n".join([
            "# comment",
            "garbage",
            "v1|NVIDIA GB300|152|bc1|128|2",                  # too few fields
            "v2|NVIDIA GB300|152|bc1|128|2|0|40.0",           # unknown version
            "v1|NVIDIA GB300|152|dxt9|128|2|0|40.0",          # unknown codec
            "v1|NVIDIA GB300|152|bc1|96|2|0|40.0",            # threads the kernels do not run
            "v1|NVIDIA GB300|152|bc1|128|4|1|40.0",           # 4 blocks a thread only without a resident grid
            "v1|NVIDIA GB300|152|both|512|4|0|40.0",          # the two-codec pass takes 1 or 2 blocks a thread
            "v1|NVIDIA GB300|152|etc1s|512|2|2|fast",         # time not a number
            "v1|NVIDIA GB300|15x|etc1s|512|2|2|40.0",         # SM count not a number
            "v1|NVIDIA GB300|152|etc1s|-512|2|2|40.0",
            "v1|NVIDIA GB300|152|etc1s|256|2|2|0",            # no time
            "v1|NVIDIA GB300|152|etc1s|128|1|2|47.5",         # the only valid line
        ]) + "\n")
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_BC1) is None
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_BOTH) is None
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_ETC1S) == (128, 1, 2)
    # storing keeps the other lines it cannot parse out of the way of lookups, and the valid one
    assert g.tile_cache_store(cache, *GB300, g.CODEC_BC1, (128, 2, 0), 41.0) == g.OK
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_ETC1S) == (128, 1, 2)
    assert g.tile_cache_lookup(cache, *GB300, g.CODEC_BC1) == (128, 2, 0)


def test_store_rejects_bad_entries_and_a_disabled_cache(cache):
    assert g.tile_cache_store(cache, *GB300, g.CODEC_BC1, (96, 2, 0), 40.0) == g.ERR_INVALID
    assert g.tile_cache_store(cache, *GB300, 3, (128, 2, 0), 40.0) == g.ERR_INVALID
    assert g.tile_cache_store(cache, *GB300, g.CODEC_BC1, (128, 2, 0), 0.0) == g.ERR_INVALID
    assert g.tile_cache_store(cache, "", 152, g.CODEC_BC1, (128, 2, 0), 40.0) == g.ERR_INVALID
    assert g.tile_cache_store("", *GB300, g.CODEC_BC1, (128, 2, 0), 40.0) == g.ERR_INVALID
    assert not os.path.exists(cache)
    # a name with the field separator is stored with it replaced, and found again under the same name
    assert g.tile_cache_store(cache, "odd|name", 8, g.CODEC_BC1, (256, 1, 0), 9.0) == g.OK
    assert g.tile_cache_lookup(cache, "odd|name", 8, g.CODEC_BC1) == (256, 1, 0)


def test_path_setting_environment_and_default(cache):
    """The explicit path wins; None falls back to $GOOFY_TILE_CACHE, then
    $XDG_CACHE_HOME, then $HOME (checked in child processes with their own
    environment)."""
    assert g.set_tile_cache_path(cache) == g.OK and g.tile_cache_path() == cache
    assert g.tile_cache_store(None, *GB300, g.CODEC_BC1, (256, 2, 0), 44.0) == g.OK  # NULL path: the one in use
    assert g.tile_cache_lookup(None, *GB300, g.CODEC_BC1) == (256, 2, 0)
    assert g.set_tile_cache_path("") == g.OK and g.tile_cache_path() == ""
    assert g.tile_cache_lookup(None, *GB300, g.CODEC_BC1) is None  # disabled
    code = "import goofy_gb300 as g; print(g.tile_cache_path())"
    base = {k: v for k, v in os.environ.items() if k not in ("GOOFY_TILE_CACHE", "XDG_CACHE_HOME", "HOME")}
    cases = [({"GOOFY_TILE_CACHE": "/x/t.txt", "XDG_CACHE_HOME": "/c", "HOME": "/h"}, "/x/t.txt"),
             ({"GOOFY_TILE_CACHE": "", "HOME": "/h"}, ""),
             ({"XDG_CACHE_HOME": "/c", "HOME": "/h"}, "/c/goofy_gb300/tiles.txt"),
             ({"HOME": "/h"}, "/h/.cache/goofy_gb300/tiles.txt")]
    for env, want in cases:
        out = subprocess.run([sys.executable, "-c", code], env=dict(base, **env), cwd=ROOT, capture_output=True,
                             text=True, check=True).stdout.strip()
        assert out == want, (env, out)
