"""Batched encoder (one persistent launch over many images of uneven sizes):
every image's output equals the oracle's, with graph replay on and off,
after autotuning, at the full mixed-batch size, and the argument checks."""
import ctypes

import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu
GUARD = 64


def _upload(torch, img, stride, offset):
    h = img.shape[0]
    rows = np.zeros((h, stride), np.uint8)
    rows[:, :img.shape[1]] = img
    buf = torch.zeros(h * stride + offset + 64, dtype=torch.uint8, device="cuda")
    buf[offset:offset + h * stride] = torch.from_numpy(rows.reshape(-1)).cuda()
    return buf, rows


def make_mixed(torch, rng, n_textures=40, max_side=512):
    """Textures with mip chains, mixed codecs, padded / unaligned strides."""
    items = []
    for t in range(n_textures):
        w = int(4 << rng.integers(2, int(np.log2(max_side)) - 1))
        h = int(4 << rng.integers(2, int(np.log2(max_side)) - 1))
        if t % 7 == 3 and t % 3 != 0:
            w += 4 * int(rng.integers(1, 5))  # ragged width (w % 16 != 0); no mip chain for these
        codec = int(rng.integers(0, 2))
        img = workloads.scene(w, h, 1000 + t)
        levels = workloads.mip_chain(w, h) if t % 3 == 0 else [(w, h)]
        cur, cw, ch = img, w, h
        for lv, (lw, lh) in enumerate(levels):
            if lv:
                cur, cw, ch = workloads.downsample(cur, cw, ch)
            extra = [0, 16, 4, 44][(t + lv) % 4]
            offset = [0, 16, 4, 0][(t * 3 + lv) % 4]
            stride = 4 * lw + extra
            buf, rows = _upload(torch, np.ascontiguousarray(cur[:, :4 * lw]), stride, offset)
            n = g.out_size(lw, lh)
            dst = torch.full((n + 2 * GUARD,), 0x5A, dtype=torch.uint8, device="cuda")
            items.append(dict(src=buf, offset=offset, rows=rows, w=lw, h=lh, stride=stride, codec=codec, dst=dst,
                              n=n))
    # edge cases: empty image between others, single block, one-block-wide column
    for (w, h) in ((0, 0), (4, 4), (4, 64), (64, 4)):
        img = workloads.scene(max(w, 4), max(h, 4), 77)[:max(h, 0), :4 * w] if w else np.zeros((0, 0), np.uint8)
        stride = 4 * max(w, 4)
        buf, rows = _upload(torch, img if w else np.zeros((4, 16), np.uint8), stride, 0)
        n = g.out_size(w, h)
        dst = torch.full((n + 2 * GUARD,), 0x5A, dtype=torch.uint8, device="cuda")
        items.insert(len(items) // 2, dict(src=buf, offset=0, rows=rows, w=w, h=h, stride=stride, codec=1, dst=dst,
                                            n=n))
    return items


def descriptors(items):
    return [(it["src"].data_ptr() + it["offset"], it["dst"].data_ptr() + GUARD, it["w"], it["h"], it["stride"],
             it["codec"]) for it in items]


def check(torch, items):
    torch.cuda.synchronize()
    for it in items:
        out = it["dst"].cpu().numpy()
        assert (out[:GUARD] == 0x5A).all() and (out[GUARD + it["n"]:] == 0x5A).all(), "write outside output"
        if it["n"] == 0:
            continue
        want = oracle.encode(it["codec"], it["rows"], it["w"], it["h"], stride=it["stride"])
        np.testing.assert_array_equal(out[GUARD:GUARD + it["n"]], want, err_msg="%dx%d codec %d stride %d" % (
            it["w"], it["h"], it["codec"], it["stride"]))


def reset(items):
    for it in items:
        it["dst"].fill_(0x5A)


@pytest.fixture(scope="module")
def mixed(cuda):
    return make_mixed(cuda, np.random.default_rng(7))


def test_batch_matches_oracle_graphs_on_and_off(cuda, mixed):
    b = g.Batch(len(mixed) + 8)
    try:
        stream = cuda.cuda.current_stream().cuda_stream
        for graphs in (True, False, True):
            b.set_graphs(graphs)
            reset(mixed)
            assert b.encode(descriptors(mixed), stream) == g.OK, g.last_error()
            check(cuda, mixed)
    finally:
        b.close()


def test_graph_replay_with_new_pointers(cuda, mixed):
    """Same shape, different destinations: the replayed graph reads the new
    descriptors; alternating slots must not mix batches up."""
    b = g.Batch(len(mixed))
    try:
        stream = cuda.cuda.current_stream().cuda_stream
        second = [dict(it, dst=cuda.full_like(it["dst"], 0x5A)) for it in mixed]
        for _ in range(3):
            reset(mixed)
            reset(second)
            assert b.encode(descriptors(mixed), stream) == g.OK
            assert b.encode(descriptors(second), stream) == g.OK
            check(cuda, mixed)
            check(cuda, second)
    finally:
        b.close()


@pytest.mark.parametrize("tile", [(128, 1, 64), (256, 2, 256), (512, 2, 2048), (512, 1, 32),
                                  (128, 1, 128, 1), (128, 2, 256, 1), (256, 1, 256, 1), (512, 2, 1024, 1)])
def test_batch_tiles(cuda, mixed, tile):
    b = g.Batch(len(mixed))
    try:
        assert b.set_tile(*tile) == g.OK
        reset(mixed)
        assert b.encode(descriptors(mixed), cuda.cuda.current_stream().cuda_stream) == g.OK
        check(cuda, mixed)
    finally:
        b.close()


@pytest.mark.parametrize("count", [1, 2, 63, 64, 65])
def test_pipelined_small_batches_pass_descriptors_inline(cuda, mixed, count):
    """A pipelined batch of at most 64 images passes its descriptors as the
    kernel's parameter instead of uploading them (65 takes the upload); both
    give every image's own blocks, with graphs on and off."""
    assert len(mixed) > 65
    items = mixed[:count]
    b = g.Batch(len(mixed))
    try:
        stream = cuda.cuda.current_stream().cuda_stream
        for tile in ((512, 2, 1024, 1), (128, 1, 128, 1)):
            assert b.set_tile(*tile) == g.OK
            for graphs in (True, False):
                b.set_graphs(graphs)
                reset(items)
                assert b.encode(descriptors(items), stream) == g.OK, g.last_error()
                check(cuda, items)
    finally:
        b.close()
    assert g.pipeline_timeouts() == 0


def test_batch_autotune(cuda, mixed):
    b = g.Batch(len(mixed))
    try:
        tile, us = b.autotune(descriptors(mixed), reps=3)
        assert tile[0] in (128, 256, 512) and tile[1] in (1, 2) and us > 0
        assert b.get_tile() == tile
        reset(mixed)
        assert b.encode(descriptors(mixed), cuda.cuda.current_stream().cuda_stream) == g.OK
        check(cuda, mixed)
    finally:
        b.close()


def test_batch_argument_checks(cuda, mixed):
    b = g.Batch(4)
    try:
        d = descriptors(mixed[:6])
        assert b.encode(d) == g.ERR_TOO_LARGE
        bad = list(d[0])
        bad[5] = 3
        assert b.encode([tuple(bad)]) == g.ERR_INVALID
        bad = list(d[1])
        bad[1] += 4  # dst not 8-byte aligned
        assert b.encode([tuple(bad)]) == g.ERR_ALIGNMENT
        bad = list(d[1])
        bad[2] = 6
        assert b.encode([tuple(bad)]) == g.ERR_WIDTH
        assert b.set_tile(256, 2, 48) == g.ERR_INVALID
        assert b.set_tile(256, 1, 512, 1) == g.ERR_INVALID  # a pipelined unit is one stage: threads * bpt
        assert b.set_tile(256, 1, 256, 2) == g.ERR_INVALID
        assert b.encode([]) == g.OK
    finally:
        b.close()


def test_full_mixed_batch_1000_textures(cuda):
    """The 1000-texture workload (sizes 64..2048, 20% with mip chains, codecs
    50/50) in one launch, bit-exact against the oracle for every level."""
    levels = workloads.texture_batch(1000)
    total = sum(lv["width"] * lv["height"] for lv in levels)
    assert 3e8 < total < 8e8
    arena_in = cuda.empty(sum(lv["pixels"].size for lv in levels) + 256 * len(levels), dtype=cuda.uint8,
                          device="cuda")
    arena_out = cuda.zeros(sum(g.out_size(lv["width"], lv["height"]) for lv in levels), dtype=cuda.uint8,
                           device="cuda")
    descs, off_in, off_out = [], 0, 0
    for lv in levels:
        px = lv["pixels"]
        arena_in[off_in:off_in + px.size] = cuda.from_numpy(np.ascontiguousarray(px).reshape(-1)).cuda()
        n = g.out_size(lv["width"], lv["height"])
        descs.append((arena_in.data_ptr() + off_in, arena_out.data_ptr() + off_out, lv["width"], lv["height"],
                      px.strides[0], lv["codec"]))
        lv["out"] = (off_out, n)
        off_in += (px.size + 255) // 256 * 256
        off_out += n
    outs = []
    b = g.Batch(len(levels))
    try:
        for tile in (None, (512, 2, 1024, 1)):  # the default tile, then the bulk-copy pipeline
            if tile:
                assert b.set_tile(*tile) == g.OK
            arena_out.zero_()
            assert b.encode(descs, cuda.cuda.current_stream().cuda_stream) == g.OK, g.last_error()
            cuda.cuda.synchronize()
            outs.append(arena_out.cpu().numpy())
    finally:
        b.close()
    assert g.pipeline_timeouts() == 0
    for lv in levels:
        o, n = lv["out"]
        want = oracle.encode(lv["codec"], lv["pixels"], lv["width"], lv["height"], threads=0 if n > 65536 else 1)
        for out in outs:
            np.testing.assert_array_equal(out[o:o + n], want)


@pytest.mark.parametrize("tile", [(512, 2, 1024, 1), (256, 1, 256, 1)])
def test_pipelined_batches_keep_stream_order(cuda, tile):
    """Pipelined batch launches (programmatic dependent launch, and an L2
    prefetch of their first rows before the dependency wait) back to back on
    one stream with an image kernel, each touching memory the previous launch
    reads or writes, without synchronisation:
      X (image kernel) writes blocks into P;
      A (batch) encodes P's bytes as an image (reads what X wrote) into Q,
        and `img` into R;
      B (batch) overwrites `img`, which A read;
      C (batch) encodes again into R, which A wrote."""
    w, h = 1024, 512
    img = workloads.scene(w, h, 8)
    other = workloads.stress(w, h, 9)
    n = g.out_size(w, h)
    st = cuda.cuda.current_stream().cuda_stream
    src = cuda.from_numpy(img.reshape(-1)).cuda()
    oth = cuda.from_numpy(other.reshape(-1)).cuda()
    p = cuda.zeros(n, dtype=cuda.uint8, device="cuda")  # X's blocks (256 KiB), read by A as a 256x256 RGBA image
    q = cuda.zeros(g.out_size(256, 256), dtype=cuda.uint8, device="cuda")
    r = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
    b = g.Batch(4)
    try:
        assert b.set_tile(*tile) == g.OK
        cuda.cuda.synchronize()
        assert g.compress_device(g.CODEC_ETC1S, p.data_ptr(), src.data_ptr(), w, h, 4 * w, st) == g.OK      # X
        assert b.encode([(p, q, 256, 256, 1024, g.CODEC_BC1), (src, r, w, h, 4 * w, g.CODEC_BC1)], st) == g.OK  # A
        assert b.encode([(oth, src, w, h, 4 * w, g.CODEC_ETC1S)], st) == g.OK                              # B
        assert b.encode([(oth, r, w, h, 4 * w, g.CODEC_ETC1S)], st) == g.OK                                # C
        cuda.cuda.synchronize()
    finally:
        b.close()
    x_blocks = oracle.encode(g.CODEC_ETC1S, img, w, h)
    np.testing.assert_array_equal(p.cpu().numpy(), x_blocks)
    np.testing.assert_array_equal(q.cpu().numpy(),
                                  oracle.encode(g.CODEC_BC1, x_blocks.reshape(256, 1024), 256, 256))
    want_b = oracle.encode(g.CODEC_ETC1S, other, w, h)
    np.testing.assert_array_equal(src[:n].cpu().numpy(), want_b)
    np.testing.assert_array_equal(r.cpu().numpy(), want_b)
