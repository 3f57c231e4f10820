"""The kernels' per-block arithmetic (goofy_gb300/csrc/block_codec.cuh and
block_decode.cuh), compiled for the CPU with emulated intrinsics, against the
golden vectors and the oracle.  Catches formulation errors before any GPU run."""
import numpy as np
import pytest

import oracle
from goofy_gb300 import workloads
from tests.host_emu import build as emu_build


@pytest.fixture(scope="module")
def emu(built):
    return emu_build.load()


def _encode(emu, codec, img, w, h):
    out = np.zeros((w // 4) * (h // 4) * 8, np.uint8)
    assert emu.host_emu_encode(codec, out.ctypes.data, img.ctypes.data, w, h, img.strides[0]) == 0
    return out


@pytest.mark.parametrize("name,codec", [("bc1", 0), ("etc1s", 1)])
def test_golden(emu, golden, name, codec):
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    np.testing.assert_array_equal(_encode(emu, codec, golden["kat_input"], w, h), golden["kat_" + name])
    np.testing.assert_array_equal(_encode(emu, codec, workloads.scene(256, 256, 0), 256, 256), golden["cfg0_" + name])
    np.testing.assert_array_equal(_encode(emu, codec, workloads.stress(256, 256, 2), 256, 256),
                                  golden["stress_" + name])


@pytest.mark.parametrize("seed", range(4))
def test_random_vs_oracle(emu, seed):
    rng = np.random.default_rng(seed)
    w, h = 256, 128
    amp = [255, 40, 6, 1][seed]
    base = rng.integers(0, 256, (h // 4, w // 4, 1, 1, 4))
    img = np.clip(base + rng.integers(-amp, amp + 1, (h // 4, w // 4, 4, 4, 4)), 0, 255)
    img = np.ascontiguousarray(img.astype(np.uint8).transpose(0, 2, 1, 3, 4).reshape(h, 4 * w))
    for codec in (0, 1):
        np.testing.assert_array_equal(_encode(emu, codec, img, w, h), oracle.encode(codec, img, w, h))


def test_edge_blocks_vs_oracle(emu):
    """Blocks whose channel bounds sit at or next to 0, 127/128 and 255: the
    brightness mid and the thresholds reach the ends of their ranges (mid 0 /
    255, qt 96, a mean pushed past 0 or 255 by the correction)."""
    rng = np.random.default_rng(5)
    w, h = 1024, 256
    edges = np.array([0, 1, 2, 3, 8, 120, 127, 128, 135, 247, 252, 253, 254, 255])
    n = (h // 4) * (w // 4)
    lo = edges[rng.integers(0, len(edges), (n, 1, 4))]
    hi = edges[rng.integers(0, len(edges), (n, 1, 4))]
    lo, hi = np.minimum(lo, hi), np.maximum(lo, hi)
    # per pixel: one of the bounds (most), or a value between them
    pick = rng.integers(0, 3, (n, 16, 4))
    mid = lo + ((hi - lo + 1) * rng.random((n, 16, 4))).astype(np.int64)
    px = np.where(pick == 0, lo, np.where(pick == 1, hi, np.minimum(mid, hi)))
    # a quarter of the blocks: all pixels at one bound but one at the other,
    # which pulls the mean farthest from the brightness mid
    odd = rng.integers(0, 16, n)
    one = np.arange(16)[None, :] == odd[:, None]
    first = rng.integers(0, 2, n).astype(bool)[:, None, None]
    lone = np.where(one[:, :, None], np.where(first, hi, lo), np.where(first, lo, hi))
    sel = (np.arange(n) % 4 == 0)[:, None, None]
    px = np.where(sel, lone, px)
    img = px.reshape(h // 4, w // 4, 4, 4, 4).transpose(0, 2, 1, 3, 4).reshape(h, 4 * w).astype(np.uint8)
    img = np.ascontiguousarray(img)
    for codec in (0, 1):
        np.testing.assert_array_equal(_encode(emu, codec, img, w, h), oracle.encode(codec, img, w, h))
    # the two-codec pass on the same blocks
    bc1, etc = _encode_both(emu, img, w, h)
    np.testing.assert_array_equal(bc1, oracle.encode(0, img, w, h))
    np.testing.assert_array_equal(etc, oracle.encode(1, img, w, h))


def _encode_both(emu, img, w, h):
    n = (w // 4) * (h // 4) * 8
    out = np.zeros(2 * n, np.uint8)
    assert emu.host_emu_encode(2, out.ctypes.data, img.ctypes.data, w, h, img.strides[0]) == 0
    return out[:n], out[n:]


def test_both_codecs_in_one_pass(emu, golden):
    """encode_both (shared lanes, extents and luma sums) gives each codec's
    own blocks: golden vectors, random blocks of every spread and the edge
    cases of the oracle tests."""
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    bc1, etc = _encode_both(emu, golden["kat_input"], w, h)
    np.testing.assert_array_equal(bc1, golden["kat_bc1"])
    np.testing.assert_array_equal(etc, golden["kat_etc1s"])
    for key, img in (("cfg0", workloads.scene(256, 256, 0)), ("stress", workloads.stress(256, 256, 2))):
        bc1, etc = _encode_both(emu, img, 256, 256)
        np.testing.assert_array_equal(bc1, golden[key + "_bc1"])
        np.testing.assert_array_equal(etc, golden[key + "_etc1s"])
    rng = np.random.default_rng(9)
    for amp in (255, 40, 6, 1, 0):
        img = rng.integers(0, 256, (64, 4 * 128)).astype(np.int64)
        img = np.clip(img - img % 64 + rng.integers(-amp, amp + 1, img.shape), 0, 255).astype(np.uint8)
        bc1, etc = _encode_both(emu, img, 128, 64)
        np.testing.assert_array_equal(bc1, oracle.encode(0, img, 128, 64))
        np.testing.assert_array_equal(etc, oracle.encode(1, img, 128, 64))


def _decode(emu, codec, blocks, w, h):
    img = np.zeros((h, 4 * w), np.uint8)
    bad = emu.host_emu_decode(codec, np.ascontiguousarray(blocks).ctypes.data, w, h, img.ctypes.data, 4 * w)
    return img, bad


@pytest.mark.parametrize("codec", [0, 1])
def test_decoder_random_blocks_vs_oracle(emu, codec):
    """Random 64-bit blocks reach every mode: BC1 in both endpoint orders,
    ETC1 individual / differential (in and out of range) with both flips."""
    rng = np.random.default_rng(11 + codec)
    w, h = 512, 256
    blocks = rng.integers(0, 256, (w // 4) * (h // 4) * 8, dtype=np.uint8)
    got, bad = _decode(emu, codec, blocks, w, h)
    want, want_bad = oracle.decode(codec, blocks, w, h)
    np.testing.assert_array_equal(got, want)
    assert bad == want_bad
    if codec == 1:
        assert 0 < bad < (w // 4) * (h // 4)


def test_decoder_etc1s_shaped_blocks_vs_oracle(emu):
    """Random ETC1s-shaped blocks (differential mode, zero deltas, one table
    for both halves, either flip) take the decoder's fast path; individual-
    mode blocks with equal halves and differential blocks with a non-zero
    delta or two tables take the general one.  All equal the oracle."""
    rng = np.random.default_rng(23)
    w, h = 256, 256
    n = (w // 4) * (h // 4)
    c5 = rng.integers(0, 32, (n, 3))
    table = rng.integers(0, 8, n)
    kind = np.arange(n) % 4  # 0, 1: ETC1s-shaped; 2: a non-zero delta; 3: two tables
    delta = np.where(kind[:, None] == 2, rng.integers(1, 8, (n, 3)), 0)
    table2 = np.where(kind == 3, (table + 1 + rng.integers(0, 7, n)) % 8, table)
    flip = rng.integers(0, 2, n)
    w0 = ((c5[:, 0] << 27) | (delta[:, 0] << 24) | (c5[:, 1] << 19) | (delta[:, 1] << 16) | (c5[:, 2] << 11) |
          (delta[:, 2] << 8) | (table << 5) | (table2 << 2) | 2 | flip).astype(np.uint64)
    w1 = rng.integers(0, 1 << 32, n, dtype=np.uint64)
    be = ((w0 << np.uint64(32)) | w1).astype(">u8")  # the block's 8 bytes, big-endian
    blocks = np.frombuffer(be.tobytes(), np.uint8).copy()
    got, bad = _decode(emu, 1, blocks, w, h)
    want, want_bad = oracle.decode(1, blocks, w, h)
    np.testing.assert_array_equal(got, want)
    assert bad == want_bad


@pytest.mark.parametrize("name,codec", [("bc1", 0), ("etc1s", 1)])
def test_decoder_on_encoder_output(emu, golden, name, codec):
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    got, bad = _decode(emu, codec, golden["kat_" + name], w, h)
    want, _ = oracle.decode(codec, golden["kat_" + name], w, h)
    np.testing.assert_array_equal(got, want)
    assert bad == 0


def test_two_level_average_identity_over_every_pair_of_sums():
    """block_codec.cuh's avg4_x4 takes two rounding averages in one step:
    avg(avg(a, b), avg(c, d)) = (s + t + 2 - (s & t & 1)) >> 2 with
    s = a + b + 1, t = c + d + 1.  Both sides depend on a, b, c, d only
    through a + b and c + d, so every pair of sums 0..510 covers every input;
    the top level of the mean runs the same identity on multiples of 4."""
    import numpy as np

    ab = np.arange(511, dtype=np.int64)[:, None]
    cd = np.arange(511, dtype=np.int64)[None, :]
    want = (((ab + 1) >> 1) + ((cd + 1) >> 1) + 1) >> 1
    s, t = ab + 1, cd + 1
    np.testing.assert_array_equal((s + t + 2 - (s & t & 1)) >> 2, want)
    # scaled by 4: columns c (multiples of 4 up to 1020), 16 * avg(avg(c0, c1), avg(c2, c3))
    s4, t4 = 4 * ab + 4, 4 * cd + 4
    np.testing.assert_array_equal((s4 + t4 + 8 - (s4 & t4 & 4)) & ~15, 16 * want)
