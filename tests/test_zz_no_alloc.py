"""goofy_gpu_batch_encode_noalloc: the batch entry point for callers that may
not allocate while they encode (its scratch is a fixed device array inside
the library).  Its output must equal the allocating batch entry point's
(goofy_gpu_batch_encode), bit for bit, on two calls in a row -- the second
call proves the shared scratch (work counter, descriptor tables) is reset
between calls.  Named to be collected last; it also passes on its own in a
fresh process."""
import numpy as np
import pytest

import goofy_gb300 as g
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu


def _images(torch, seed, n):
    """n textures of mixed sizes, codecs and strides, resident on the device."""
    rng = np.random.default_rng(seed)
    items = []
    for t in range(n):
        w = int(4 << rng.integers(1, 8))
        h = int(4 << rng.integers(1, 8))
        codec = int(rng.integers(0, 2))
        stride = 4 * w + [0, 16, 4][t % 3]
        img = np.zeros((h, stride), np.uint8)
        img[:, :4 * w] = workloads.scene(w, h, seed * 1000 + t)
        src = torch.from_numpy(img.reshape(-1)).cuda()
        n_out = g.out_size(w, h)
        items.append(dict(src=src, w=w, h=h, stride=stride, codec=codec, n=n_out,
                          dst_a=torch.full((n_out,), 0x11, dtype=torch.uint8, device="cuda"),
                          dst_b=torch.full((n_out,), 0x22, dtype=torch.uint8, device="cuda")))
    return items


def _descs(items, key):
    return [(it["src"].data_ptr(), it[key].data_ptr(), it["w"], it["h"], it["stride"], it["codec"]) for it in items]


def test_noalloc_matches_batch_entry_point_twice(cuda):
    stream = cuda.cuda.current_stream().cuda_stream
    ref = g.Batch(g.NOALLOC_MAX_IMAGES)
    try:
        for call, (seed, n) in enumerate([(1, 60), (2, 37)]):
            items = _images(cuda, seed, n)
            rc = g.batch_encode_noalloc(_descs(items, "dst_a"), stream)
            assert rc == g.OK, (call, g.status_string(rc), g.last_error())
            assert ref.encode(_descs(items, "dst_b"), stream) == g.OK, g.last_error()
            cuda.cuda.synchronize()
            for it in items:
                np.testing.assert_array_equal(it["dst_a"].cpu().numpy(), it["dst_b"].cpu().numpy())
    finally:
        ref.close()


def test_noalloc_rejects_more_than_its_maximum(cuda):
    items = _images(cuda, 3, 1)
    descs = _descs(items, "dst_a") * (g.NOALLOC_MAX_IMAGES + 1)
    assert g.batch_encode_noalloc(descs) == g.ERR_TOO_LARGE
    assert "at most %d images" % g.NOALLOC_MAX_IMAGES in g.last_error()
    cuda.cuda.synchronize()
    assert (items[0]["dst_a"].cpu().numpy() == 0x11).all()  # nothing was launched
