"""GPU parity of the two-codec pass (goofy_gpu_compress_both_*): one read of
the image writes the BC1 blocks of goofy::compressDXT1 and the ETC1s blocks
of goofy::compressETC1, each bit-exact against the oracle and the golden
vectors -- every tile shape, ragged sizes, word-aligned rows, the host paths
with pinned and pageable buffers, and the full 8192x8192 workload."""
import ctypes
import hashlib

import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu

TILES = [(t, b, p) for p in (0, 1, 2) for t in (128, 256, 512) for b in (1, 2)]
GUARD = 256


def both_device(torch, img, w, h, stride=None, src_offset=0, tile=None):
    """Upload `img`, run the two-codec pass, return (BC1, ETC1s) with the
    guard bands around both outputs checked."""
    stride = stride or img.strides[0]
    rows = np.zeros((h, stride), np.uint8)
    rows[:, :img.shape[1]] = img[:, :min(img.shape[1], stride)]
    src = torch.zeros(h * stride + src_offset + 64, dtype=torch.uint8, device="cuda")
    src[src_offset:src_offset + h * stride] = torch.from_numpy(rows.reshape(-1)).cuda()
    n = g.out_size(w, h)
    dst = torch.full((2 * n + 3 * GUARD,), 0xA5, dtype=torch.uint8, device="cuda")
    if tile is not None:
        before = g.get_tile(g.CODEC_BOTH)
        assert g.set_tile(g.CODEC_BOTH, *tile) == g.OK
    try:
        rc = g.compress_both_device(dst.data_ptr() + GUARD, dst.data_ptr() + 2 * GUARD + n,
                                    src.data_ptr() + src_offset, w, h, stride, torch.cuda.current_stream().cuda_stream)
    finally:
        if tile is not None:
            g.set_tile(g.CODEC_BOTH, *before)
    assert rc == g.OK, (rc, g.status_string(rc), g.last_error())
    torch.cuda.synchronize()
    out = dst.cpu().numpy()
    for a, b in ((0, GUARD), (GUARD + n, 2 * GUARD + n), (2 * GUARD + 2 * n, 3 * GUARD + 2 * n)):
        assert (out[a:b] == 0xA5).all(), "write outside the outputs"
    return out[GUARD:GUARD + n], out[2 * GUARD + n:2 * GUARD + 2 * n]


@pytest.mark.parametrize("tile", TILES)
def test_golden_vectors_every_tile(cuda, golden, tile):
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    bc1, etc = both_device(cuda, golden["kat_input"], w, h, tile=tile)
    np.testing.assert_array_equal(bc1, golden["kat_bc1"])
    np.testing.assert_array_equal(etc, golden["kat_etc1s"])
    for key, img in (("cfg0", workloads.scene(256, 256, 0)), ("stress", workloads.stress(256, 256, 2))):
        bc1, etc = both_device(cuda, img, 256, 256, tile=tile)
        np.testing.assert_array_equal(bc1, golden[key + "_bc1"])
        np.testing.assert_array_equal(etc, golden[key + "_etc1s"])


@pytest.mark.parametrize("w,h", [(4, 4), (12, 8), (36, 36), (260, 8), (1028, 20), (4, 256), (2052, 4)])
def test_ragged_sizes(cuda, w, h):
    rng = np.random.default_rng(w * 1000 + h + 7)
    img = rng.integers(0, 256, (h, 4 * w), dtype=np.uint8)
    want = (oracle.encode(0, img, w, h), oracle.encode(1, img, w, h))
    for tile in ((256, 1, 0), (128, 2, 0), (128, 1, 2), (512, 2, 2)):
        bc1, etc = both_device(cuda, img, w, h, tile=tile)
        np.testing.assert_array_equal(bc1, want[0])
        np.testing.assert_array_equal(etc, want[1])


@pytest.mark.parametrize("extra,offset", [(0, 0), (48, 16), (4, 0), (0, 4), (260, 4)])
def test_strides_and_alignment(cuda, extra, offset):
    """Word-aligned rows take the register-loading kernel whatever the tile."""
    w, h = 72, 24
    img = workloads.scene(w, h, 13)
    bc1, etc = both_device(cuda, img, w, h, stride=4 * w + extra, src_offset=offset)
    np.testing.assert_array_equal(bc1, oracle.encode(0, img, w, h))
    np.testing.assert_array_equal(etc, oracle.encode(1, img, w, h))


@pytest.mark.parametrize("path", [g.HOST_PATH_AUTO, g.HOST_PATH_STAGED, g.HOST_PATH_DIRECT])
def test_host_paths_pinned_and_pageable(cuda, path):
    """goofy_gpu_compress_both_host over a 64 MiB image with a padded stride
    (several bands on the staged path), pageable and pinned buffers."""
    w, h = 4096, 4096
    stride = 4 * w + 64
    img = np.zeros((h, stride), np.uint8)
    img[:, :4 * w] = workloads.scene(w, h, 22, period_scale=16, rects=256, threads=0)
    want = [oracle.encode(c, img, w, h, stride=stride, threads=0) for c in (0, 1)]
    assert g.set_host_path(path) == g.OK
    n = g.out_size(w, h)
    p_in, p_out = g.host_alloc(h * stride), g.host_alloc(2 * n)
    try:
        bc1, etc = np.zeros(n, np.uint8), np.zeros(n, np.uint8)
        assert g.compress_both_host(bc1, etc, img, w, h, stride) == g.OK, g.last_error()
        np.testing.assert_array_equal(bc1, want[0])
        np.testing.assert_array_equal(etc, want[1])
        assert p_in and p_out
        src = np.ctypeslib.as_array((ctypes.c_uint8 * (h * stride)).from_address(p_in))
        dst = np.ctypeslib.as_array((ctypes.c_uint8 * (2 * n)).from_address(p_out))
        src[:] = img.reshape(-1)
        dst[:] = 0
        assert g.compress_both_host(p_out, p_out + n, p_in, w, h, stride) == g.OK, g.last_error()
        np.testing.assert_array_equal(dst[:n], want[0])
        np.testing.assert_array_equal(dst[n:], want[1])
    finally:
        g.set_host_path(g.HOST_PATH_AUTO)
        g.host_free(p_in)
        g.host_free(p_out)


def test_full_size_scene_8192(cuda):
    """The 8192x8192 workload: both outputs equal the two single-codec
    launches (themselves pinned to the oracle by the parity tests) for each
    tile, repeatably, with no pipeline time-outs."""
    w = h = 8192
    img = workloads.scene(w, h, 1, period_scale=32, rects=2048, threads=0)
    src = cuda.from_numpy(img.reshape(-1)).cuda()
    n = g.out_size(w, h)
    st = cuda.cuda.current_stream().cuda_stream
    single = []
    for c in (g.CODEC_BC1, g.CODEC_ETC1S):
        d = cuda.empty(n, dtype=cuda.uint8, device="cuda")
        assert g.compress_device(c, d.data_ptr(), src.data_ptr(), w, h, 4 * w, st) == g.OK
        single.append(d)
    cuda.cuda.synchronize()
    want = [hashlib.sha256(d.cpu().numpy().tobytes()).hexdigest() for d in single]
    # the first 64 block rows against the oracle directly
    for c in (0, 1):
        np.testing.assert_array_equal(single[c][:64 * (w // 4) * 8].cpu().numpy(),
                                      oracle.encode(c, np.ascontiguousarray(img[:256]), w, 256, threads=0))
    out = cuda.empty(2 * n, dtype=cuda.uint8, device="cuda")
    before = g.get_tile(g.CODEC_BOTH)
    try:
        for tile in (before, (512, 1, 2), (256, 2, 2), (128, 2, 0)):
            assert g.set_tile(g.CODEC_BOTH, *tile) == g.OK
            for _ in range(2):
                out.fill_(0)
                assert g.compress_both_device(out.data_ptr(), out.data_ptr() + n, src.data_ptr(), w, h, 4 * w,
                                              st) == g.OK
                cuda.cuda.synchronize()
                got = out.cpu().numpy()
                assert [hashlib.sha256(got[:n].tobytes()).hexdigest(),
                        hashlib.sha256(got[n:].tobytes()).hexdigest()] == want, tile
    finally:
        g.set_tile(g.CODEC_BOTH, *before)
    assert g.pipeline_timeouts() == 0


def test_autotune_the_two_codec_pass(cuda):
    """GOOFY_CODEC_BOTH autotunes the two-codec pass over a buffer holding
    both outputs; the installed tile is one the pass runs, and its outputs
    stay bit-exact."""
    w = h = 1024
    img = workloads.scene(w, h, 17, period_scale=4, rects=64)
    n = g.out_size(w, h)
    src = cuda.from_numpy(img.reshape(-1)).cuda()
    out = cuda.zeros(2 * n, dtype=cuda.uint8, device="cuda")
    before = g.get_tile(g.CODEC_BOTH)
    try:
        tile, us = g.autotune(g.CODEC_BOTH, out, src, w, h, 4 * w, reps=3)
        assert g.get_tile(g.CODEC_BOTH) == tile and tile[1] <= 2 and tile[2] != 1 and us > 0
        assert g.compress_both_device(out, out.data_ptr() + n, src, w, h, 4 * w,
                                      cuda.cuda.current_stream().cuda_stream) == g.OK
        cuda.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got[:n], oracle.encode(0, img, w, h))
        np.testing.assert_array_equal(got[n:], oracle.encode(1, img, w, h))
    finally:
        g.set_tile(g.CODEC_BOTH, *before)
