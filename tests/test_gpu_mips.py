"""Device mip chains equal the host chain (the workload generator's 2x2
box filter) bit for bit, and a whole texture -- mips made on the device,
all levels encoded in one batch launch -- equals the oracle level by level."""
import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu


def _host_chain(img, w, h):
    out, cur, cw, ch = [img], img, w, h
    for lw, lh in workloads.mip_chain(w, h)[1:]:
        cur, cw, ch = workloads.downsample(cur, cw, ch)
        out.append(cur)
    return out


@pytest.mark.parametrize("w,h", [(4, 4), (8, 4), (8, 8), (16, 16), (64, 64), (256, 32), (16, 1024), (4096, 64),
                                 (2048, 2048)])
def test_device_mips_equal_host_chain(cuda, w, h):
    img = workloads.scene(w, h, w + h)
    host = _host_chain(img, w, h)
    d_src = cuda.from_numpy(img.reshape(-1)).cuda()
    nbytes = max(g.lib().goofy_gpu_mip_arena_bytes(w, h), 256)
    arena = cuda.zeros(nbytes + 256, dtype=cuda.uint8, device="cuda")
    base = arena.data_ptr() + (-arena.data_ptr()) % 256
    levels = g.generate_mips(d_src, w, h, 4 * w, base, nbytes, cuda.cuda.current_stream().cuda_stream)
    cuda.cuda.synchronize()
    assert len(levels) == len(host) == g.lib().goofy_gpu_mip_count(w, h)
    flat = arena.cpu().numpy()
    off0 = base - arena.data_ptr()
    for (ptr, lw, lh, stride), want in zip(levels[1:], host[1:]):
        o = off0 + (ptr - base)
        got = flat[o:o + stride * lh].reshape(lh, stride)[:, :4 * lw]
        np.testing.assert_array_equal(got, want)


def test_mips_argument_checks(cuda):
    d = cuda.zeros(64 * 64 * 4, dtype=cuda.uint8, device="cuda")
    assert g.lib().goofy_gpu_mip_count(12, 16) == 0
    with pytest.raises(RuntimeError):
        g.generate_mips(d, 12, 16, 48, d, 1 << 16)


@pytest.mark.parametrize("codec", [0, 1])
def test_texture_with_device_mips_in_one_batch(cuda, codec):
    w, h = 512, 128
    img = workloads.scene(w, h, 77)
    d_src = cuda.from_numpy(img.reshape(-1)).cuda()
    nbytes = g.lib().goofy_gpu_mip_arena_bytes(w, h)
    arena = cuda.empty(nbytes + 256, dtype=cuda.uint8, device="cuda")
    base = arena.data_ptr() + (-arena.data_ptr()) % 256
    stream = cuda.cuda.current_stream().cuda_stream
    levels = g.generate_mips(d_src, w, h, 4 * w, base, nbytes, stream)
    outs = [cuda.zeros(g.out_size(lw, lh), dtype=cuda.uint8, device="cuda") for _, lw, lh, _ in levels]
    b = g.Batch(len(levels))
    try:
        assert b.encode([(p, o.data_ptr(), lw, lh, s, codec) for (p, lw, lh, s), o in zip(levels, outs)],
                        stream) == g.OK
        cuda.cuda.synchronize()
    finally:
        b.close()
    for (p, lw, lh, s), o, ref in zip(levels, outs, _host_chain(img, w, h)):
        np.testing.assert_array_equal(o.cpu().numpy(), oracle.encode(codec, ref, lw, lh))
