"""Oracle package -- TEST INFRASTRUCTURE ONLY.

``load()`` returns the ctypes handle of the C restatement (goofy_oracle.c);
``load_ref()`` the reference encoder compiled from its own header with its
SSE2 path (None where the reference tree is absent or the host is not
x86-64); ``load_ref_scalar()`` the reference encoder's own scalar path, built
from the header copy without goofy_tc.h:16 (None where that copy was never
generated); ``ref_encoder()`` the best of these for a CPU baseline.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU legs use these; the product
package never imports this module.
"""
import ctypes
import os

from .build import ORACLE_SO, REF_SCALAR_SO, REF_SO

_VP = ctypes.c_void_p
_U = ctypes.c_uint
_oracle = None
_ref = None
_ref_scalar = None


def load():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            from .build import build
            build()
        lib = ctypes.CDLL(ORACLE_SO)
        lib.oracle_encode_block.restype = None
        lib.oracle_encode_block.argtypes = [ctypes.c_int, _VP, ctypes.c_size_t, _VP]
        for name in ("oracle_compress", "oracle_compress_any"):
            fn = getattr(lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_int, _VP, _VP, _U, _U, _U]
        lib.oracle_compress_mt.restype = ctypes.c_int
        lib.oracle_compress_mt.argtypes = [ctypes.c_int, _VP, _VP, _U, _U, _U, ctypes.c_int]
        lib.oracle_decode_block.restype = ctypes.c_int
        lib.oracle_decode_block.argtypes = [ctypes.c_int, _VP, _VP]
        lib.oracle_decode_image.restype = ctypes.c_long
        lib.oracle_decode_image.argtypes = [ctypes.c_int, _VP, _U, _U, _VP, _U]
        lib.oracle_sq_error.restype = None
        lib.oracle_sq_error.argtypes = [_VP, _U, _VP, _U, _U, _U, _VP]
        lib.oracle_mse_psnr.restype = None
        lib.oracle_mse_psnr.argtypes = [_VP, _U, _VP, _U, _U, _U, _VP]
        lib.oracle_psnr_rgb.restype = ctypes.c_double
        lib.oracle_psnr_rgb.argtypes = [_VP, _U, _U]
        lib.goofy_synth_scene.restype = ctypes.c_int
        lib.goofy_synth_scene.argtypes = [_VP, _U, _U, _U, ctypes.c_uint64, _U, _U, ctypes.c_int]
        _oracle = lib
    return _oracle


def load_ref():
    """The reference itself (x86-64 with the reference tree present), else None."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        lib = ctypes.CDLL(REF_SO)
        lib.ref_compress.restype = ctypes.c_int
        lib.ref_compress.argtypes = [ctypes.c_int, _VP, _VP, _U, _U, _U]
        lib.ref_compress_mt.restype = ctypes.c_int
        lib.ref_compress_mt.argtypes = [ctypes.c_int, _VP, _VP, _U, _U, _U, ctypes.c_int]
        lib.ref_decode_block.restype = None
        lib.ref_decode_block.argtypes = [ctypes.c_int, _VP, _VP]
        lib.ref_png_decode.restype = ctypes.c_uint
        lib.ref_png_decode.argtypes = [_VP, ctypes.c_size_t, _VP, ctypes.c_size_t, ctypes.POINTER(_U),
                                       ctypes.POINTER(_U)]
        _ref = lib
    return _ref


def load_ref_scalar():
    """The reference encoder's scalar path (GOOFY_SSE2 undefined), else None."""
    global _ref_scalar
    if _ref_scalar is None and os.path.exists(REF_SCALAR_SO):
        lib = ctypes.CDLL(REF_SCALAR_SO)
        lib.ref_compress.restype = ctypes.c_int
        lib.ref_compress.argtypes = [ctypes.c_int, _VP, _VP, _U, _U, _U]
        lib.ref_compress_mt.restype = ctypes.c_int
        lib.ref_compress_mt.argtypes = [ctypes.c_int, _VP, _VP, _U, _U, _U, ctypes.c_int]
        _ref_scalar = lib
    return _ref_scalar


def ref_encoder():
    """(compress_mt function, kind, label) of the reference's own CPU encoder
    for a baseline: its SSE2 path where built, else its scalar path, else the
    oracle port (kind "port")."""
    ref = load_ref()
    if ref is not None:
        return ref.ref_compress_mt, "reference", "reference goofy_tc.h, SSE2 path"
    ref = load_ref_scalar()
    if ref is not None:
        return (ref.ref_compress_mt, "reference",
                "reference goofy_tc.h, its portable scalar path (GOOFY_SSE2 undefined; SSE2 is x86-only)")
    return load().oracle_compress_mt, "port", "oracle port of the reference encoder (reference not built here)"


def scene(w, h, seed, period_scale=1, rects=8, threads=0):
    """The synthetic scene (goofy_gb300/csrc/synth.c, compiled into the oracle
    library) as an (h, 4w) RGBA8 array with 256-byte aligned rows."""
    import numpy as np

    raw = np.empty(h * 4 * w + 256, np.uint8)
    off = (-raw.ctypes.data) % 256
    img = raw[off:off + h * 4 * w].reshape(h, 4 * w)
    if load().goofy_synth_scene(img.ctypes.data, w, h, 4 * w, seed, period_scale, rects, threads) != 0:
        raise ValueError("goofy_synth_scene failed")
    return img


def encode(codec, img, width, height, stride=None, threads=1, any_width=True):
    """Oracle output for an RGBA8 numpy image (rows of `stride` bytes)."""
    import numpy as np

    stride = stride or img.strides[0]
    out = np.zeros((width // 4) * (height // 4) * 8, np.uint8)
    lib = load()
    if threads != 1:
        rc = lib.oracle_compress_mt(codec, out.ctypes.data, img.ctypes.data, width, height, stride, threads)
        rc = 0 if rc > 0 else rc
    elif any_width:
        rc = lib.oracle_compress_any(codec, out.ctypes.data, img.ctypes.data, width, height, stride)
    else:
        rc = lib.oracle_compress(codec, out.ctypes.data, img.ctypes.data, width, height, stride)
    if rc != 0:
        raise ValueError("oracle rejected the image: %d" % rc)
    return out


def decode(codec, blocks, width, height):
    """Oracle decode of (width/4)*(height/4) blocks into an RGBA8 image."""
    import numpy as np

    img = np.zeros((height, 4 * width), np.uint8)
    bad = load().oracle_decode_image(codec, np.ascontiguousarray(blocks).ctypes.data, width, height, img.ctypes.data,
                                     4 * width)
    return img, bad


def sq_error(a, b, width, height):
    """Per-channel sums of squared differences (uint64[4]) of two RGBA8 images."""
    import numpy as np

    sums = np.zeros(4, np.uint64)
    load().oracle_sq_error(a.ctypes.data, a.strides[0], b.ctypes.data, b.strides[0], width, height, sums.ctypes.data)
    return sums


MSE_PSNR_FIELDS = ("mse_r", "mse_g", "mse_b", "mse_a", "mse_max", "mse_rgb", "mse_y",
                   "psnr_r", "psnr_g", "psnr_b", "psnr_a", "psnr_min", "psnr_rgb", "psnr_y")


def mse_psnr(a, b, width, height):
    """The harness's getMsePsnr of two RGBA8 images, as a dict."""
    import numpy as np

    out = np.zeros(14, np.float64)
    load().oracle_mse_psnr(a.ctypes.data, a.strides[0], b.ctypes.data, b.strides[0], width, height, out.ctypes.data)
    return dict(zip(MSE_PSNR_FIELDS, out.tolist()))


def psnr_rgb(sums, width, height):
    import numpy as np

    s = np.ascontiguousarray(sums, dtype=np.uint64)
    return load().oracle_psnr_rgb(s.ctypes.data, width, height)


def ref_png_decode(data, max_pixels=1 << 26):
    """The harness's PNG loader (lodepng::decode to RGBA8) on PNG bytes:
    (error, rgba rows (h, 4w), w, h); None without the reference library."""
    import numpy as np

    lib = load_ref()
    if lib is None:
        return None
    buf = ctypes.create_string_buffer(bytes(data), len(data))
    out = np.zeros(4 * max_pixels, np.uint8)
    w, h = _U(), _U()
    err = lib.ref_png_decode(buf, len(data), out.ctypes.data, out.nbytes, ctypes.byref(w), ctypes.byref(h))
    if err:
        return err, None, 0, 0
    return 0, out[:4 * w.value * h.value].reshape(h.value, 4 * w.value).copy(), w.value, h.value
