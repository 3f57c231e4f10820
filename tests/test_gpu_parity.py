"""GPU parity: the sm_103a kernels through the C ABI, bit-exact against the
oracle and the reference's golden vectors -- every tile shape, ragged sizes,
strides and alignments, the host (drop-in) pipeline with pinned and pageable
buffers, and the full-size workloads."""
import ctypes
import hashlib

import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu

CODECS = [("bc1", g.CODEC_BC1), ("etc1s", g.CODEC_ETC1S)]
TILES = [(t, b, p) for p in (0, 1, 2) for t in (128, 256, 512) for b in (1, 2, 4) if not (p and b == 4)]
GUARD = 256


def device_encode(torch, codec, img, w, h, stride=None, src_offset=0, tile=None):
    """Upload `img` (h rows, `stride` bytes each) at `src_offset` bytes into a
    device buffer, encode, and return the output (guard bands checked)."""
    stride = stride or img.strides[0]
    rows = np.zeros((h, stride), np.uint8)
    rows[:, :img.shape[1]] = img[:, :min(img.shape[1], stride)]
    src = torch.zeros(h * stride + src_offset + 64, dtype=torch.uint8, device="cuda")
    src[src_offset:src_offset + h * stride] = torch.from_numpy(rows.reshape(-1)).cuda()
    n = g.out_size(w, h)
    dst = torch.full((n + 2 * GUARD,), 0xA5, dtype=torch.uint8, device="cuda")
    if tile is not None:
        before = g.get_tile(codec)
        assert g.set_tile(codec, *tile) == g.OK
    try:
        rc = g.compress_device(codec, dst.data_ptr() + GUARD, src.data_ptr() + src_offset, w, h, stride,
                               torch.cuda.current_stream().cuda_stream)
    finally:
        if tile is not None:
            g.set_tile(codec, *before)
    assert rc == g.OK, (rc, g.status_string(rc), g.last_error())
    torch.cuda.synchronize()
    out = dst.cpu().numpy()
    assert (out[:GUARD] == 0xA5).all() and (out[GUARD + n:] == 0xA5).all(), "write outside the output"
    return out[GUARD:GUARD + n]


@pytest.mark.parametrize("name,codec", CODECS)
@pytest.mark.parametrize("tile", TILES)
def test_golden_vectors_every_tile(cuda, golden, name, codec, tile):
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    np.testing.assert_array_equal(device_encode(cuda, codec, golden["kat_input"], w, h, tile=tile),
                                  golden["kat_" + name])
    cfg0 = workloads.scene(256, 256, 0)
    np.testing.assert_array_equal(device_encode(cuda, codec, cfg0, 256, 256, tile=tile), golden["cfg0_" + name])
    st = workloads.stress(256, 256, 2)
    np.testing.assert_array_equal(device_encode(cuda, codec, st, 256, 256, tile=tile), golden["stress_" + name])


@pytest.mark.parametrize("name,codec", CODECS)
@pytest.mark.parametrize("w,h", [(4, 4), (8, 4), (12, 8), (20, 12), (36, 36), (100, 16), (260, 8), (1028, 20),
                                 (4, 256), (2052, 4)])
def test_ragged_sizes(cuda, name, codec, w, h):
    rng = np.random.default_rng(w * 1000 + h)
    img = rng.integers(0, 256, (h, 4 * w), dtype=np.uint8)
    want = oracle.encode(codec, img, w, h)
    for tile in ((256, 1, 0), (128, 4, 0), (256, 2, 1), (128, 1, 2), (512, 2, 2)):
        np.testing.assert_array_equal(device_encode(cuda, codec, img, w, h, tile=tile), want)


@pytest.mark.parametrize("name,codec", CODECS)
@pytest.mark.parametrize("extra,offset", [(0, 0), (16, 0), (48, 16), (4, 0), (0, 4), (12, 8), (260, 4)])
def test_strides_and_alignment(cuda, name, codec, extra, offset):
    """16-byte aligned base and stride use the vector loads, 4-byte aligned
    ones the word loads; both must give the same bits."""
    w, h = 72, 24
    img = workloads.scene(w, h, 11)
    stride = 4 * w + extra
    want = oracle.encode(codec, img, w, h)
    np.testing.assert_array_equal(device_encode(cuda, codec, img, w, h, stride=stride, src_offset=offset), want)


@pytest.mark.parametrize("name,codec", CODECS)
@pytest.mark.parametrize("path", [g.HOST_PATH_AUTO, g.HOST_PATH_STAGED, g.HOST_PATH_DIRECT])
def test_host_path_pinned_and_pageable(cuda, name, codec, path):
    """goofy_gpu_compress_host / goofy::compress*: 64 MiB image through the
    staged band pipeline or the direct path, pageable and pinned buffers,
    padded stride."""
    assert g.set_host_path(path) == g.OK
    try:
        _host_path_case(codec)
    finally:
        g.set_host_path(g.HOST_PATH_AUTO)


def _host_path_case(codec):
    w, h = 4096, 4096
    stride = 4 * w + 64
    img = np.zeros((h, stride), np.uint8)
    img[:, :4 * w] = workloads.scene(w, h, 21, period_scale=16, rects=256, threads=0)
    want = oracle.encode(codec, img, w, h, stride=stride, threads=0)
    out = np.zeros(g.out_size(w, h), np.uint8)
    fn = g.compressDXT1 if codec == g.CODEC_BC1 else g.compressETC1
    assert fn(out, img, w, h, stride) == 0, g.last_error()
    np.testing.assert_array_equal(out, want)
    # pinned buffers take the direct-DMA branch
    n_in, n_out = h * stride, g.out_size(w, h)
    p_in, p_out = g.host_alloc(n_in), g.host_alloc(n_out)
    assert p_in and p_out
    try:
        src = np.ctypeslib.as_array((ctypes.c_uint8 * n_in).from_address(p_in))
        dst = np.ctypeslib.as_array((ctypes.c_uint8 * n_out).from_address(p_out))
        src[:] = img.reshape(-1)
        dst[:] = 0
        assert g.compress_host(codec, p_out, p_in, w, h, stride) == g.OK, g.last_error()
        np.testing.assert_array_equal(dst, want)
        # ragged width through the host path (w % 16 != 0 is fine off the drop-in)
        assert g.compress_host(codec, p_out, p_in, w - 4, h, stride) == g.OK
        np.testing.assert_array_equal(dst[:g.out_size(w - 4, h)],
                                      oracle.encode(codec, img, w - 4, h, stride=stride, threads=0))
    finally:
        g.host_free(p_in)
        g.host_free(p_out)


@pytest.mark.parametrize("name,codec", CODECS)
def test_full_size_scene_8192(cuda, name, codec):
    """The 8192x8192 workload (256 MiB in, 32 MiB out) bit-exact against the
    multi-threaded oracle, and repeatable."""
    w = h = 8192
    img = workloads.scene(w, h, 1, period_scale=32, rects=2048, threads=0)
    want = oracle.encode(codec, img, w, h, threads=0)
    src = cuda.from_numpy(img.reshape(-1)).cuda()
    dst = cuda.empty(g.out_size(w, h), dtype=cuda.uint8, device="cuda")
    before = g.get_tile(codec)
    try:
        for tile in (before, (256, 1, 2), (512, 2, 2), (128, 2, 2)):
            assert g.set_tile(codec, *tile) == g.OK
            for _ in range(2):
                dst.fill_(0)
                assert g.compress_device(codec, dst.data_ptr(), src.data_ptr(), w, h, 4 * w,
                                         cuda.cuda.current_stream().cuda_stream) == g.OK
                cuda.cuda.synchronize()
                got = dst.cpu().numpy()
                assert hashlib.sha256(got.tobytes()).hexdigest() == hashlib.sha256(want.tobytes()).hexdigest(), tile
    finally:
        g.set_tile(codec, *before)
    assert g.pipeline_timeouts() == 0


@pytest.mark.parametrize("name,codec", CODECS)
def test_full_size_stress_4096(cuda, name, codec):
    w = h = 4096
    img = workloads.stress(w, h, 2)
    want = oracle.encode(codec, img, w, h, threads=0)
    np.testing.assert_array_equal(device_encode(cuda, codec, img, w, h), want)
    # every quarter on its own equals the corresponding columns of the whole
    q = w // 4
    full = want.reshape(h // 4, w // 4, 8)
    for k in range(4):
        part = device_encode(cuda, codec, np.ascontiguousarray(img[:, 4 * k * q:4 * (k + 1) * q]), q, h)
        np.testing.assert_array_equal(part.reshape(h // 4, q // 4, 8), full[:, k * q // 4:(k + 1) * q // 4])


def test_image_larger_than_4_gib(cuda):
    """A 32772x32768 image (4,295,491,584 bytes, past 2^32, rows of 131,088
    bytes, 8193 blocks a row so every row of tiles ends in a one-block tile):
    the single-codec kernels (bulk-copy ring and register-loading grid), the
    two-codec pass and a one-image batch all match the oracle.  Each row's
    content differs (a band of noise XOR a per-row byte), so a block read
    from a wrapped 32-bit offset would not match."""
    w, h = 32772, 32768
    stride = 4 * w
    assert stride * h > 1 << 32
    rng = np.random.default_rng(42)
    band = rng.integers(0, 256, (64, stride), dtype=np.uint8)
    img = np.tile(band, (h // 64, 1))
    img ^= ((np.arange(h, dtype=np.uint64) * 2654435761) >> np.uint64(7)).astype(np.uint8)[:, None]
    want = [oracle.encode(c, img, w, h, threads=0) for c in (g.CODEC_BC1, g.CODEC_ETC1S)]
    src = cuda.from_numpy(img.reshape(-1)).cuda()
    del img
    n = g.out_size(w, h)
    out = cuda.empty(2 * n, dtype=cuda.uint8, device="cuda")
    stream = cuda.cuda.current_stream().cuda_stream

    def check(k, label):
        cuda.cuda.synchronize()
        got = out[k * n:(k + 1) * n].cpu().numpy()
        assert np.array_equal(got, want[k]), label

    for c in (g.CODEC_BC1, g.CODEC_ETC1S):
        before = g.get_tile(c)
        try:
            for tile in (before, (128, 2, 0)):
                assert g.set_tile(c, *tile) == g.OK
                out.fill_(0)
                assert g.compress_device(c, out[c * n:].data_ptr(), src.data_ptr(), w, h, stride, stream) == g.OK
                check(c, (c, tile))
        finally:
            g.set_tile(c, *before)
    out.fill_(0)
    assert g.compress_both_device(out.data_ptr(), out[n:].data_ptr(), src.data_ptr(), w, h, stride, stream) == g.OK
    check(0, "both, bc1")
    check(1, "both, etc1s")
    b = g.Batch(2)
    try:
        out.fill_(0)
        assert b.encode([(src, out[:n], w, h, stride, g.CODEC_BC1), (src, out[n:], w, h, stride, g.CODEC_ETC1S)],
                        stream) == g.OK
        check(0, "batch, bc1")
        check(1, "batch, etc1s")
    finally:
        b.close()
    assert g.pipeline_timeouts() == 0


def test_concurrent_kernels_bit_exact(cuda):
    """The two codecs on two streams at once, one through the bulk-copy
    pipeline and the other through a register-loading kernel sharing its SMs
    (whose global loads crowd the load/store queues), each output equal to the
    oracle's.  A compute warp that released its ring stage before its shared
    loads had read it once let the stage's next tile overwrite rows of the
    current one in exactly this setting."""
    w = h = 8192
    img = workloads.scene(w, h, 1, period_scale=32, rects=2048, threads=0)
    want = [cuda.from_numpy(oracle.encode(c, img, w, h, threads=0)).cuda() for c in (0, 1)]
    src = [cuda.from_numpy(img.reshape(-1)).cuda() for _ in range(2)]
    outs = [cuda.empty(g.out_size(w, h), dtype=cuda.uint8, device="cuda") for _ in range(2)]
    streams = [cuda.cuda.current_stream(), cuda.cuda.Stream()]
    before = [g.get_tile(c) for c in (0, 1)]
    g.pipeline_timeouts(reset=True)
    try:
        for pipe in (1, 0):  # the codec on the bulk-copy kernel
            for pipe_tile in ((128, 2, 2), (128, 1, 2), (512, 1, 2), (512, 2, 2), (256, 1, 2)):
                for grid_tile in ((128, 2, 0), (128, 1, 0)):
                    assert g.set_tile(pipe, *pipe_tile) == g.OK
                    assert g.set_tile(1 - pipe, *grid_tile) == g.OK
                    for _ in range(4):
                        for o in outs:
                            o.zero_()
                        ev = cuda.cuda.Event()
                        ev.record(streams[0])
                        streams[1].wait_event(ev)
                        for c in (pipe, 1 - pipe):  # the pipelined kernel first, so it is resident when the other starts
                            assert g.compress_device(c, outs[c].data_ptr(), src[c].data_ptr(), w, h, 4 * w,
                                                     streams[c].cuda_stream) == g.OK
                        cuda.cuda.synchronize()
                        for c in (0, 1):
                            assert cuda.equal(outs[c], want[c]), (pipe, pipe_tile, grid_tile, c)
    finally:
        for c in (0, 1):
            g.set_tile(c, *before[c])
    assert g.pipeline_timeouts() == 0


def test_back_to_back_launches_keep_stream_order(cuda):
    """Encoder launches back to back on one stream without synchronisation,
    each one touching memory the previous one reads or writes.  The encoders
    may be scheduled while the previous kernel drains (programmatic dependent
    launch), but must not touch global memory before it is done: B overwrites
    the source A reads, C encodes again into the blocks A wrote, D reads C's
    blocks (decode + error sums)."""
    w = h = 2048
    img = workloads.scene(w, h, 5, threads=0)
    other = workloads.stress(w, h, 6)
    n = g.out_size(w, h)
    st = cuda.cuda.current_stream().cuda_stream
    before = [g.get_tile(c) for c in (0, 1)]
    try:
        for tiles in ((before[0], before[1]), ((128, 1, 0), (128, 2, 2)), ((512, 1, 2), (128, 2, 0))):
            for c in (0, 1):
                assert g.set_tile(c, *tiles[c]) == g.OK
            for ca, cb in ((0, 1), (1, 0), (1, 1)):
                work = cuda.from_numpy(img.reshape(-1)).cuda()
                oth = cuda.from_numpy(other.reshape(-1)).cuda()
                out = cuda.empty(n, dtype=cuda.uint8, device="cuda")
                sums = cuda.zeros(6, dtype=cuda.int64, device="cuda")
                cuda.cuda.synchronize()
                assert g.compress_device(ca, out.data_ptr(), work.data_ptr(), w, h, 4 * w, st) == g.OK      # A
                assert g.compress_device(cb, work.data_ptr(), oth.data_ptr(), w, h, 4 * w, st) == g.OK      # B
                first = out.clone()
                assert g.compress_device(cb, out.data_ptr(), oth.data_ptr(), w, h, 4 * w, st) == g.OK       # C
                assert g.block_error_device(cb, out, oth, w, h, 4 * w, sums, st) == g.OK                    # D
                cuda.cuda.synchronize()
                np.testing.assert_array_equal(first.cpu().numpy(), oracle.encode(ca, img, w, h))
                want_b = oracle.encode(cb, other, w, h)
                np.testing.assert_array_equal(work[:n].cpu().numpy(), want_b)
                np.testing.assert_array_equal(out.cpu().numpy(), want_b)
                dec, _ = oracle.decode(cb, want_b, w, h)
                np.testing.assert_array_equal(sums.cpu().numpy()[:4].astype(np.uint64),
                                              oracle.sq_error(other, dec, w, h))
    finally:
        for c in (0, 1):
            g.set_tile(c, *before[c])


def test_pipeline_reports_no_timeouts(cuda):
    """The bulk-copy pipeline's bounded waits never expire in a healthy run."""
    g.pipeline_timeouts(reset=True)
    img = workloads.scene(1024, 512, 3)
    for codec in (0, 1):
        for tile in ((128, 1, 2), (256, 2, 2), (512, 1, 2)):
            np.testing.assert_array_equal(device_encode(cuda, codec, img, 1024, 512, tile=tile),
                                          oracle.encode(codec, img, 1024, 512))
    assert g.pipeline_timeouts() == 0


def test_bounded_wait_gives_up_and_the_context_stays_usable(cuda, golden):
    """A pipeline wait on a barrier that nothing completes (no copy, no
    arrival) gives up after its one-second limit, raises the abort flag and
    counts once; the kernel returns and the next launches are bit-exact."""
    before = g.pipeline_timeouts()
    rc, ms = g.selftest_bounded_wait()
    assert rc == g.OK, g.last_error()
    assert 900 <= ms <= 10000, ms
    assert g.pipeline_timeouts() == before  # the self-test counts in its own counter
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    for name, codec in CODECS:
        for tile in ((512, 2, 2), (128, 2, 0)):
            np.testing.assert_array_equal(device_encode(cuda, codec, golden["kat_input"], w, h, tile=tile),
                                          golden["kat_" + name])
