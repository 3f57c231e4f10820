"""Test-only build of the kernel's block arithmetic for the CPU (g++ with the
CUDA intrinsics emulated in host_emulation.h)."""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SO = os.path.join(HERE, "_build", "libblock_codec_host.so")
SOURCES = [os.path.join(HERE, "block_codec_host.cpp"), os.path.join(HERE, "host_emulation.h"),
           os.path.join(ROOT, "goofy_gb300", "csrc", "block_codec.cuh"),
           os.path.join(ROOT, "goofy_gb300", "csrc", "block_decode.cuh")]


def load():
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    if not os.path.exists(SO) or any(os.path.getmtime(s) > os.path.getmtime(SO) for s in SOURCES):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-DGOOFY_HOST_EMULATION",
                               "-I", HERE, "-I", os.path.join(ROOT, "goofy_gb300", "csrc"), "-o", SO, SOURCES[0]])
    lib = ctypes.CDLL(SO)
    lib.host_emu_encode.restype = ctypes.c_int
    lib.host_emu_encode.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint,
                                    ctypes.c_uint]
    lib.host_emu_decode.restype = ctypes.c_long
    lib.host_emu_decode.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p,
                                    ctypes.c_uint]
    return lib
