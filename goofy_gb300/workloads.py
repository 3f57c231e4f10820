"""Synthetic workloads with the shapes and value distributions of the
benchmark configurations (the reference benchmarks photographs that cannot be
shipped here; libgoofy_synth.so generates stand-ins deterministically on any
host).

* ``scene(w, h, seed, period_scale, rects)`` -- gradient + 4-octave value
  noise + rectangles; 256x256 seed 0 (8 rectangles) is the small plain case,
  8192x8192 seed 1 with periods x32 and 2048 rectangles the large one.
* ``stress(w, h, seed)`` -- the four degenerate quarters (4096x4096 seed 2).
* ``texture_batch(n)`` -- the mixed batch of n textures (sizes 64..2048,
  20% with full mip chains, BC1 / ETC1s 50/50).
"""
import ctypes

import numpy as np

from . import synth_lib


def _aligned_empty(h, stride, align=256):
    raw = np.empty(h * stride + align, np.uint8)
    off = (-raw.ctypes.data) % align
    return raw[off:off + h * stride].reshape(h, stride)


def scene(w, h, seed, period_scale=1, rects=8, stride=None, threads=0, out=None):
    stride = stride or 4 * w
    img = out if out is not None else _aligned_empty(h, stride)
    rc = synth_lib().goofy_synth_scene(img.ctypes.data, w, h, stride, seed, period_scale, rects, threads)
    if rc != 0:
        raise ValueError("goofy_synth_scene failed")
    return img


def stress(w, h, seed, stride=None):
    stride = stride or 4 * w
    img = _aligned_empty(h, stride)
    if synth_lib().goofy_synth_stress(img.ctypes.data, w, h, stride, seed) != 0:
        raise ValueError("goofy_synth_stress failed")
    return img


def downsample(img, w, h):
    """Next mip level of an RGBA8 image (2x2 box, sizes clamped at 4)."""
    dw, dh = max(w // 2, 4), max(h // 2, 4)
    out = _aligned_empty(dh, 4 * dw)
    synth_lib().goofy_synth_downsample(out.ctypes.data, 4 * dw, img.ctypes.data, w, h, img.strides[0])
    return out, dw, dh


def texture_spec(index):
    w, h, m, c = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_int(), ctypes.c_int()
    synth_lib().goofy_synth_texture_spec(index, ctypes.byref(w), ctypes.byref(h), ctypes.byref(m), ctypes.byref(c))
    return w.value, h.value, bool(m.value), c.value


def mip_chain(w, h):
    """Level sizes down to 4x4 (each axis halves, clamped at 4)."""
    sizes = [(w, h)]
    while sizes[-1] != (4, 4):
        cw, ch = sizes[-1]
        sizes.append((max(cw // 2, 4), max(ch // 2, 4)))
    return sizes


def texture_batch(n, first=0, with_pixels=True):
    """List of dicts {index, level, width, height, codec, pixels} for the mixed
    batch; pixels come from scene() with seed = texture index (mips by 2x2
    box filter of the level above)."""
    out = []
    for t in range(first, first + n):
        w, h, mips, codec = texture_spec(t)
        levels = mip_chain(w, h) if mips else [(w, h)]
        img = scene(w, h, t) if with_pixels else None
        for lv, (lw, lh) in enumerate(levels):
            if lv > 0 and with_pixels:
                img, _, _ = downsample(img, levels[lv - 1][0], levels[lv - 1][1])
            out.append({"index": t, "level": lv, "width": lw, "height": lh, "codec": codec,
                        "pixels": img})
    return out
