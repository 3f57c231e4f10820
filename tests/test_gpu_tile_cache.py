"""The tile cache on a GPU: the drop-in entry point's first call installs the
tiles recorded for this GPU model (and encodes bit-exact with them), tiles
set explicitly stay, and the autotuner records its pick for the next
process."""
import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture
def cache(cuda, tmp_path):
    path = str(tmp_path / "tiles.txt")
    g.set_tile_cache_path(path)
    g.reset_tiles()
    yield path
    g.reset_tiles()
    g.set_tile_cache_path(None)


def test_dropin_installs_cached_tiles(cache):
    name, sms = g.device_key(0)
    assert name and sms > 0
    defaults = {c: g.get_tile(c) for c in (g.CODEC_BC1, g.CODEC_ETC1S)}
    cached = {g.CODEC_BC1: (256, 1, 0), g.CODEC_ETC1S: (256, 2, 2)}
    assert all(cached[c] != defaults[c] for c in cached)
    for c, t in cached.items():
        assert g.tile_cache_store(cache, name, sms, c, t, 50.0) == g.OK
    g.tile_cache_store(cache, "some other GPU", sms, g.CODEC_BOTH, (128, 1, 0), 10.0)  # not this model's
    w = h = 256
    img = workloads.scene(w, h, 0)
    for c, fn in ((g.CODEC_BC1, g.compressDXT1), (g.CODEC_ETC1S, g.compressETC1)):
        out = np.zeros(g.out_size(w, h), np.uint8)
        assert fn(out, img, w, h, 4 * w) == 0, g.last_error()
        assert g.get_tile(c) == cached[c]  # installed by the first call
        np.testing.assert_array_equal(out, oracle.encode(c, img, w, h))
    assert g.get_tile(g.CODEC_BOTH) == (512, 2, 2)  # no entry for this model: the default stays


def test_explicit_tiles_win_over_the_cache(cache):
    name, sms = g.device_key(0)
    g.tile_cache_store(cache, name, sms, g.CODEC_BC1, (256, 1, 0), 50.0)
    g.tile_cache_store(cache, name, sms, g.CODEC_ETC1S, (256, 2, 2), 50.0)
    assert g.set_tile(g.CODEC_BC1, 128, 1, 0) == g.OK
    assert g.load_tile_cache(0) == 1  # ETC1s only
    assert g.get_tile(g.CODEC_BC1) == (128, 1, 0) and g.get_tile(g.CODEC_ETC1S) == (256, 2, 2)


def test_autotune_records_its_pick(cache, cuda):
    name, sms = g.device_key(0)
    w = h = 1024
    img = workloads.scene(w, h, 2)
    src = cuda.from_numpy(img.reshape(-1)).cuda()
    dst = cuda.empty(g.out_size(w, h), dtype=cuda.uint8, device="cuda")
    tile, us = g.autotune(g.CODEC_ETC1S, dst.data_ptr(), src.data_ptr(), w, h, 4 * w, reps=2)
    assert us > 0 and g.get_tile(g.CODEC_ETC1S) == tile
    assert g.tile_cache_lookup(cache, name, sms, g.CODEC_ETC1S) == tile
    cuda.cuda.synchronize()
    np.testing.assert_array_equal(dst.cpu().numpy(), oracle.encode(g.CODEC_ETC1S, img, w, h))


def test_pair_autotune_installs_and_records_both(cache, cuda):
    """goofy_gpu_autotune_pair: both codecs' tiles installed and recorded, and
    the alternating launches with them stay bit-exact."""
    name, sms = g.device_key(0)
    w, h = 1024, 512
    img = workloads.scene(w, h, 3)
    src = cuda.from_numpy(img.reshape(-1)).cuda()
    n = g.out_size(w, h)
    dst = cuda.empty(2 * n, dtype=cuda.uint8, device="cuda")
    t_bc1, t_etc1s, us = g.autotune_pair(dst.data_ptr(), dst.data_ptr() + n, src.data_ptr(), w, h, 4 * w, reps=2)
    assert us > 0
    assert g.get_tile(g.CODEC_BC1) == t_bc1 and g.get_tile(g.CODEC_ETC1S) == t_etc1s
    assert g.tile_cache_lookup(cache, name, sms, g.CODEC_BC1) == t_bc1
    assert g.tile_cache_lookup(cache, name, sms, g.CODEC_ETC1S) == t_etc1s
    stream = cuda.cuda.current_stream().cuda_stream
    out = cuda.zeros(2 * n, dtype=cuda.uint8, device="cuda")
    for c in (g.CODEC_BC1, g.CODEC_ETC1S):
        assert g.compress_device(c, out.data_ptr() + c * n, src.data_ptr(), w, h, 4 * w, stream) == g.OK
    cuda.cuda.synchronize()
    for c in (g.CODEC_BC1, g.CODEC_ETC1S):
        np.testing.assert_array_equal(out[c * n:(c + 1) * n].cpu().numpy(), oracle.encode(c, img, w, h))
    # overlapping outputs are refused
    assert g.lib().goofy_gpu_autotune_pair(dst.data_ptr(), dst.data_ptr() + 8, src.data_ptr(), w, h, 4 * w, 2,
                                           None, None, None) == g.ERR_INVALID
