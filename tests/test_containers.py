"""DDS / KTX containers: one level equals the reference harness's files byte
for byte (md5 of its parrot_red outputs, where the reference images exist);
mip chains carry the level count and every level in order."""
import hashlib
import os
import struct

import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from oracle.build import TEST_DATA
from goofy_gb300 import workloads

PARROT = os.path.join(TEST_DATA, "parrot_red.png")
# md5 of the reference harness's parrot_red_simd_goofy_dxt1.dds / _etc1.ktx
REF_MD5 = {0: "72e3e448ff684294a9158859101645a3", 1: "affe18054aea11c5bdbe20841a414fbc"}


def test_single_level_matches_reference_files(built):
    if not os.path.exists(PARROT):
        pytest.skip("reference test images not available on this host")
    from tests.pngread import read_png_rgba

    img, w, h = read_png_rgba(PARROT)
    for codec in (0, 1):
        blocks = oracle.encode(codec, img, w, h, any_width=False)
        assert hashlib.md5(g.container(codec, [(blocks, w, h)])).hexdigest() == REF_MD5[codec]


def test_headers_and_mip_chain(built):
    img = workloads.scene(64, 32, 3)
    levels, cur, w, h = [], img, 64, 32
    for lw, lh in workloads.mip_chain(64, 32):
        if (lw, lh) != (w, h):
            cur, w, h = workloads.downsample(cur, w, h)
        levels.append((oracle.encode(0, cur, w, h), w, h))
    dds = g.container(0, levels)
    magic, size, flags, hh, ww, linear, depth, mips = struct.unpack("<8I", dds[:32])
    assert (magic, size, flags, hh, ww, linear, depth, mips) == (0x20534444, 124, 0x000A1007, 32, 64, 1024, 1,
                                                                 len(levels))
    assert struct.unpack("<3I", dds[76:88]) == (32, 4, 0x31545844)
    body = b"".join(np.asarray(b).tobytes() for b, _, _ in levels)
    assert dds[128:] == body
    etc_levels = [(oracle.encode(1, np.zeros((lh, 4 * lw), np.uint8), lw, lh), lw, lh) for _, lw, lh in levels]
    ktx = g.container(1, etc_levels)
    assert ktx[:12] == bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])
    fields = struct.unpack("<13I", ktx[12:64])
    # endianness, glType, glTypeSize, glFormat, glInternalFormat, glBaseInternalFormat, w, h, d, arrays, faces, levels
    assert fields[0] == 0x04030201 and fields[2] == 1 and fields[4] == 0x8D64 and fields[5] == 0x1907
    assert (fields[6], fields[7], fields[10], fields[11], fields[12]) == (64, 32, 1, len(levels), 0)
    pos = 64
    for b, lw, lh in etc_levels:
        n = struct.unpack("<I", ktx[pos:pos + 4])[0]
        assert n == (lw // 4) * (lh // 4) * 8 and ktx[pos + 4:pos + 4 + n] == np.asarray(b).tobytes()
        pos += 4 + n
    assert pos == len(ktx)


def test_container_argument_checks(built):
    import ctypes

    lib = g.lib()
    w = (ctypes.c_uint32 * 1)(6)
    h = (ctypes.c_uint32 * 1)(8)
    assert lib.goofy_gpu_container_size(0, w, h, 1) == 0
    assert lib.goofy_gpu_container_size(3, w, h, 1) == 0
    w[0] = 8
    assert lib.goofy_gpu_container_size(0, w, h, 1) == 128 + 32
    assert lib.goofy_gpu_container_size(1, w, h, 1) == 64 + 4 + 32
    out = np.zeros(64, np.uint8)
    blk = np.zeros(32, np.uint8)
    ptrs = (ctypes.c_void_p * 1)(blk.ctypes.data)
    assert lib.goofy_gpu_write_container(0, ptrs, w, h, 1, out.ctypes.data, 64) == g.ERR_TOO_LARGE
