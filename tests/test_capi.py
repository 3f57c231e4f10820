"""C-ABI library checks that need no GPU: it loads, exports every function
the public headers declare, and rejects bad arguments with the documented
codes before touching CUDA (the reference's -1 / -2 included)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import goofy_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_c_functions():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not hdr.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", hdr)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        names += re.findall(r"\b(goofy_gpu_\w+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(g.LIB_PATH)
    names = declared_c_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    # the C++ drop-in (goofy_tc_gpu.h) with the reference's exact signatures
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", g.LIB_PATH], capture_output=True, text=True).stdout
    assert "goofy::compressDXT1(unsigned char*, unsigned char const*, unsigned int, unsigned int, unsigned int)" in out
    assert "goofy::compressETC1(unsigned char*, unsigned char const*, unsigned int, unsigned int, unsigned int)" in out


def test_dropin_error_codes_match_reference(built):
    img = np.zeros((64, 256), np.uint8)
    out = np.zeros(4096, np.uint8)
    for fn in (g.compressDXT1, g.compressETC1):
        assert fn(out, img, 60, 64, 256) == -1      # width % 16
        assert fn(out, img, 8, 64, 256) == -1
        assert fn(out, img, 64, 62, 256) == -2      # height % 4
        assert fn(out, img, 64, 3, 256) == -2


def test_c_abi_argument_checks(built):
    lib = g.lib()
    out = np.zeros(4096, np.uint8)
    img = np.zeros((64, 256), np.uint8)
    for codec in (0, 1):
        assert g.compress_device(codec, 16, 16, 6, 8, 64) == g.ERR_WIDTH
        assert g.compress_device(codec, 16, 16, 8, 6, 64) == g.ERR_HEIGHT
        assert g.compress_device(codec, None, 16, 8, 8, 64) == g.ERR_INVALID
        assert g.compress_device(codec, 16, 16, 8, 8, 16) == g.ERR_INVALID   # stride < 4*width
        assert g.compress_device(codec, 12, 16, 8, 8, 64) == g.ERR_ALIGNMENT  # dst not 8-byte aligned
        assert g.compress_device(codec, 16, 18, 8, 8, 64) == g.ERR_ALIGNMENT  # src not 4-byte aligned
        assert g.compress_host(codec, out, img, 62, 64, 256) == g.ERR_WIDTH
        assert g.compress_host(codec, out, None, 64, 64, 256) == g.ERR_INVALID
        assert g.compress_device(codec, 16, 16, 0, 8, 64) == g.OK  # empty image: nothing to do
    assert g.compress_device(7, 16, 16, 8, 8, 64) == g.ERR_INVALID
    assert lib.goofy_gpu_status_string(g.ERR_ALIGNMENT) == b"misaligned pointer or stride"


def test_both_codecs_argument_checks(built):
    """The two-codec pass checks what each single-codec call checks, plus its
    second output; the single-output calls refuse the two-codec id."""
    out, out2 = np.zeros(4096, np.uint8), np.zeros(4096, np.uint8)
    img = np.zeros((64, 256), np.uint8)
    assert g.compress_both_device(16, 4096, 16, 6, 8, 64) == g.ERR_WIDTH
    assert g.compress_both_device(16, 4096, 16, 8, 6, 64) == g.ERR_HEIGHT
    assert g.compress_both_device(16, None, 16, 8, 8, 64) == g.ERR_INVALID
    assert g.compress_both_device(None, 4096, 16, 8, 8, 64) == g.ERR_INVALID
    assert g.compress_both_device(16, 4096, 16, 8, 8, 16) == g.ERR_INVALID   # stride < 4*width
    assert g.compress_both_device(16, 4100, 16, 8, 8, 64) == g.ERR_ALIGNMENT  # ETC1s output not 8-byte aligned
    assert g.compress_both_device(16, 4096, 18, 8, 8, 64) == g.ERR_ALIGNMENT  # src not 4-byte aligned
    assert g.compress_both_device(16, 24, 16, 0, 8, 64) == g.OK  # empty image: nothing to do
    assert g.compress_both_device(4096, 4096 + 24, 16, 8, 8, 64) == g.ERR_INVALID  # outputs of 32 B overlap
    assert g.compress_both_device(4096 + 24, 4096, 16, 8, 8, 64) == g.ERR_INVALID
    assert g.compress_both_host(out, out[8:], img, 64, 64, 256) == g.ERR_INVALID
    assert g.compress_both_host(out, None, img, 64, 64, 256) == g.ERR_INVALID
    assert g.compress_both_host(out, out2, img, 62, 64, 256) == g.ERR_WIDTH
    assert g.compress_device(g.CODEC_BOTH, 16, 16, 8, 8, 64) == g.ERR_INVALID
    assert g.compress_host(g.CODEC_BOTH, out, img, 64, 64, 256) == g.ERR_INVALID


def test_tile_get_set(built):
    for codec in (0, 1):
        before = g.get_tile(codec)
        assert g.set_tile(codec, 512, 2, 1) == g.OK
        assert g.get_tile(codec) == (512, 2, 1)
        assert g.set_tile(codec, 256, 4, 0) == g.OK
        assert g.set_tile(codec, 256, 4, 1) == g.ERR_INVALID
        assert g.set_tile(codec, 256, 2, 2) == g.OK
        assert g.set_tile(codec, 256, 4, 2) == g.ERR_INVALID
        assert g.set_tile(codec, 256, 2, 3) == g.ERR_INVALID
        assert g.set_tile(codec, 96, 2) == g.ERR_INVALID
        assert g.set_tile(codec, 256, 3) == g.ERR_INVALID
        assert g.set_tile(codec, *before) == g.OK
    # the two-codec pass has its own tile: 1 or 2 blocks a thread
    before = g.get_tile(g.CODEC_BOTH)
    assert g.set_tile(g.CODEC_BOTH, 256, 1, 2) == g.OK and g.get_tile(g.CODEC_BOTH) == (256, 1, 2)
    assert g.set_tile(g.CODEC_BOTH, 256, 4, 0) == g.ERR_INVALID
    assert g.set_tile(g.CODEC_BOTH, *before) == g.OK
    assert g.set_tile(3, 256, 2, 0) == g.ERR_INVALID


def test_server_config_checks_before_cuda(built):
    """goofy_gpu_server_create rejects a bad config before touching CUDA."""
    cfg = g.ServerConfig()
    g.lib().goofy_gpu_server_default_config(ctypes.byref(cfg))
    assert cfg.completion == g.COMPLETION_CALLBACK and cfg.mode == g.SERVER_STAGED
    h = ctypes.c_void_p()
    for field, bad in (("completion", 2), ("mode", 5), ("quality", 2), ("max_batch_images", 0)):
        c = g.ServerConfig()
        g.lib().goofy_gpu_server_default_config(ctypes.byref(c))
        setattr(c, field, bad)
        assert g.lib().goofy_gpu_server_create(ctypes.byref(h), ctypes.byref(c)) == g.ERR_INVALID, field
        assert not h.value
