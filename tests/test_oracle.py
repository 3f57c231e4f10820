"""The oracle (C restatement) pinned against the reference's own outputs:
the golden vectors the reference produced, and -- where the reference tree
exists on this host -- the reference encoder itself on fresh inputs."""
import hashlib

import numpy as np
import pytest

import oracle
from goofy_gb300 import workloads

CODECS = [("bc1", 0), ("etc1s", 1)]


@pytest.mark.parametrize("name,codec", CODECS)
def test_oracle_matches_golden_kat(built, golden, name, codec):
    img = golden["kat_input"]
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    np.testing.assert_array_equal(oracle.encode(codec, img, w, h, any_width=False), golden["kat_" + name])


@pytest.mark.parametrize("name,codec", CODECS)
def test_oracle_matches_golden_cfg0(built, golden, name, codec):
    img = workloads.scene(256, 256, 0)
    assert hashlib.sha256(img.tobytes()).hexdigest() == str(golden["cfg0_sha256"])
    np.testing.assert_array_equal(oracle.encode(codec, img, 256, 256, any_width=False), golden["cfg0_" + name])


@pytest.mark.parametrize("name,codec", CODECS)
def test_oracle_matches_golden_stress(built, golden, name, codec):
    img = workloads.stress(256, 256, 2)
    assert hashlib.sha256(img.tobytes()).hexdigest() == str(golden["stress_sha256"])
    np.testing.assert_array_equal(oracle.encode(codec, img, 256, 256, any_width=False), golden["stress_" + name])


def test_oracle_error_codes(oracle_lib):
    buf = np.zeros(64 * 64 * 4, np.uint8)
    out = np.zeros(64 * 64 // 2, np.uint8)
    for codec in (0, 1):
        assert oracle_lib.oracle_compress(codec, out.ctypes.data, buf.ctypes.data, 60, 64, 240) == -1
        assert oracle_lib.oracle_compress(codec, out.ctypes.data, buf.ctypes.data, 64, 62, 256) == -2
        assert oracle_lib.oracle_compress_any(codec, out.ctypes.data, buf.ctypes.data, 62, 64, 248) == -1
        assert oracle_lib.oracle_compress_any(codec, out.ctypes.data, buf.ctypes.data, 60, 64, 240) == 0


def test_oracle_multithreaded_equals_single(built):
    img = workloads.scene(512, 256, 5)
    for codec in (0, 1):
        np.testing.assert_array_equal(oracle.encode(codec, img, 512, 256, threads=4),
                                      oracle.encode(codec, img, 512, 256))


def test_narrow_levels_equal_padded_reference_rows(built):
    """oracle_compress_any on a w % 16 != 0 image equals the 16-pixel padded
    image's output with the padding blocks dropped (blocks are independent)."""
    rng = np.random.default_rng(3)
    for w in (4, 8, 12, 20):
        h = 16
        img = rng.integers(0, 256, (h, 4 * w), dtype=np.uint8)
        pw = (w + 15) // 16 * 16
        pad = np.zeros((h, 4 * pw), np.uint8)
        pad[:, :4 * w] = img
        for codec in (0, 1):
            full = oracle.encode(codec, pad, pw, h, any_width=False).reshape(h // 4, pw // 4, 8)
            np.testing.assert_array_equal(oracle.encode(codec, img, w, h).reshape(h // 4, w // 4, 8),
                                          full[:, :w // 4])


def _ref_or_skip():
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("reference encoder not available on this host")
    return ref


def _aligned(img):
    buf = np.empty(img.size + 64, np.uint8)
    off = (-buf.ctypes.data) % 64
    a = buf[off:off + img.size].reshape(img.shape)
    a[...] = img
    return a


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_matches_reference_random(built, seed):
    ref = _ref_or_skip()
    rng = np.random.default_rng(100 + seed)
    w, h = 512, 256
    kinds = [rng.integers(0, 256, (h, 4 * w)),
             np.clip(rng.integers(0, 256, (h // 4, w // 4, 1, 1, 4)) + rng.integers(-9, 10, (h // 4, w // 4, 4, 4, 4)),
                     0, 255).transpose(0, 2, 1, 3, 4).reshape(h, 4 * w)]
    for img in kinds:
        img = _aligned(img.astype(np.uint8))
        for codec in (0, 1):
            want = np.zeros(w * h // 2, np.uint8)
            assert ref.ref_compress(codec, want.ctypes.data, img.ctypes.data, w, h, 4 * w) == 0
            np.testing.assert_array_equal(oracle.encode(codec, img, w, h, any_width=False), want)


def test_oracle_matches_reference_scene_and_stress_large(built):
    ref = _ref_or_skip()
    for img, w, h in ((workloads.scene(1024, 512, 7, period_scale=4, rects=64), 1024, 512),
                      (workloads.stress(1024, 1024, 2), 1024, 1024)):
        img = _aligned(img)
        for codec in (0, 1):
            want = np.zeros(w * h // 2, np.uint8)
            assert ref.ref_compress(codec, want.ctypes.data, img.ctypes.data, w, h, 4 * w) == 0
            np.testing.assert_array_equal(oracle.encode(codec, img, w, h, threads=4), want)


def test_reference_error_codes(built):
    ref = _ref_or_skip()
    img = _aligned(np.zeros((64, 256), np.uint8))
    out = np.zeros(4096, np.uint8)
    assert ref.ref_compress(0, out.ctypes.data, img.ctypes.data, 60, 64, 256) == -1
    assert ref.ref_compress(1, out.ctypes.data, img.ctypes.data, 64, 62, 256) == -2


def test_reference_scalar_path_matches_sse2_path_and_oracle(built):
    """The reference's own scalar path (the generated header copy without
    goofy_tc.h:16, the CPU baseline on hosts without SSE2) gives the blocks of
    its SSE2 path and of the oracle, block for block, and keeps the error codes."""
    scalar = oracle.load_ref_scalar()
    if scalar is None:
        pytest.skip("the scalar header copy was never generated on this host")
    ref = oracle.load_ref()
    rng = np.random.default_rng(9)
    w, h = 512, 256
    imgs = [_aligned(rng.integers(0, 256, (h, 4 * w)).astype(np.uint8)),
            _aligned(workloads.scene(w, h, 4, rects=32)), _aligned(workloads.stress(w, h, 2))]
    for img in imgs:
        for codec in (0, 1):
            got = np.zeros(w * h // 2, np.uint8)
            assert scalar.ref_compress_mt(codec, got.ctypes.data, img.ctypes.data, w, h, 4 * w, 3) == 3
            np.testing.assert_array_equal(got, oracle.encode(codec, img, w, h, any_width=False))
            if ref is not None:
                want = np.zeros_like(got)
                assert ref.ref_compress(codec, want.ctypes.data, img.ctypes.data, w, h, 4 * w) == 0
                np.testing.assert_array_equal(got, want)
    out = np.zeros(4096, np.uint8)
    assert scalar.ref_compress(0, out.ctypes.data, imgs[0].ctypes.data, 60, 64, 4 * w) == -1
    assert scalar.ref_compress(1, out.ctypes.data, imgs[0].ctypes.data, 64, 62, 4 * w) == -2


def test_oracle_scene_generator_is_the_libraries_generator(built):
    """The CPU arm of the benchmark makes its scene with the generator compiled
    into the oracle library; it equals the one the GPU arm uses."""
    np.testing.assert_array_equal(oracle.scene(768, 256, 1, period_scale=3, rects=40),
                                  workloads.scene(768, 256, 1, period_scale=3, rects=40))
