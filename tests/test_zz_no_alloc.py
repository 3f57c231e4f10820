"""goofy_gpu_batch_encode_noalloc: the batch entry point for callers that may
not allocate while they encode (its scratch is a fixed device array inside
the library).  Its output must equal the oracle's, block for block, and the
allocating batch entry point's (goofy_gpu_batch_encode), on two calls in a
row -- the second call proves the shared scratch (work counter, descriptor
tables) is reset between calls.  Also: a call of exactly its maximum image
count with empty images mixed in, and the errors it returns before
launching anything.  Named to be collected last; it also passes on its own
in a fresh process."""
import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu


def _images(torch, seed, n, sizes=(1, 8), empty_every=0):
    """n textures of mixed sizes, codecs and strides, resident on the device.
    With empty_every = k, every k-th texture is 0x0, 4x0 or 0x4 (no blocks)."""
    rng = np.random.default_rng(seed)
    items = []
    for t in range(n):
        w = int(4 << rng.integers(*sizes))
        h = int(4 << rng.integers(*sizes))
        if empty_every and t % empty_every == 0:
            w, h = [(0, 0), (4, 0), (0, 4)][(t // empty_every) % 3]
        codec = int(rng.integers(0, 2))
        stride = 4 * w + [0, 16, 4][t % 3]
        img = np.zeros((max(h, 1), max(stride, 4)), np.uint8)
        if w and h:
            img[:, :4 * w] = workloads.scene(w, h, seed * 1000 + t)
        src = torch.from_numpy(img.reshape(-1)).cuda()
        n_out = g.out_size(w, h)
        items.append(dict(img=img, src=src, w=w, h=h, stride=stride, codec=codec, n=n_out,
                          dst_a=torch.full((max(n_out, 8),), 0x11, dtype=torch.uint8, device="cuda"),
                          dst_b=torch.full((max(n_out, 8),), 0x22, dtype=torch.uint8, device="cuda")))
    return items


def _descs(items, key):
    return [(it["src"].data_ptr(), it[key].data_ptr(), it["w"], it["h"], it["stride"], it["codec"]) for it in items]


def _want(it):
    if it["n"] == 0:
        return np.zeros(0, np.uint8)
    return oracle.encode(it["codec"], it["img"], it["w"], it["h"], it["stride"])


def test_noalloc_matches_oracle_and_batch_entry_point_twice(cuda):
    stream = cuda.cuda.current_stream().cuda_stream
    ref = g.Batch(g.NOALLOC_MAX_IMAGES)
    try:
        for call, (seed, n) in enumerate([(1, 60), (2, 37)]):
            items = _images(cuda, seed, n)
            rc = g.batch_encode_noalloc(_descs(items, "dst_a"), stream)
            assert rc == g.OK, (call, g.status_string(rc), g.last_error())
            assert ref.encode(_descs(items, "dst_b"), stream) == g.OK, g.last_error()
            cuda.cuda.synchronize()
            for i, it in enumerate(items):
                got = it["dst_a"].cpu().numpy()[:it["n"]]
                np.testing.assert_array_equal(got, _want(it), err_msg="call %d image %d vs oracle" % (call, i))
                np.testing.assert_array_equal(got, it["dst_b"].cpu().numpy()[:it["n"]])
    finally:
        ref.close()


def test_noalloc_at_its_maximum_with_empty_images(cuda):
    """Exactly NOALLOC_MAX_IMAGES images, every 7th one 0x0 / 4x0 / 0x4: the
    empty ones get no work and leave their buffers alone, the rest match the
    oracle (twice, the second call with the codecs swapped)."""
    stream = cuda.cuda.current_stream().cuda_stream
    items = _images(cuda, 5, g.NOALLOC_MAX_IMAGES, sizes=(0, 5), empty_every=7)
    assert sum(it["n"] == 0 for it in items) >= 30
    for call in range(2):
        if call:
            for it in items:
                it["codec"] ^= 1
        rc = g.batch_encode_noalloc(_descs(items, "dst_a"), stream)
        assert rc == g.OK, (call, g.status_string(rc), g.last_error())
        cuda.cuda.synchronize()
        for i, it in enumerate(items):
            got = it["dst_a"].cpu().numpy()
            if it["n"] == 0:
                assert (got == 0x11).all(), (call, i)
            else:
                np.testing.assert_array_equal(got[:it["n"]], _want(it), err_msg="call %d image %d" % (call, i))


def test_noalloc_rejects_more_than_its_maximum(cuda):
    items = _images(cuda, 3, 1)
    descs = _descs(items, "dst_a") * (g.NOALLOC_MAX_IMAGES + 1)
    assert g.batch_encode_noalloc(descs) == g.ERR_TOO_LARGE
    assert "at most %d images" % g.NOALLOC_MAX_IMAGES in g.last_error()
    cuda.cuda.synchronize()
    assert (items[0]["dst_a"].cpu().numpy() == 0x11).all()  # nothing was launched


def test_noalloc_rejects_bad_arguments_before_launching(cuda):
    assert g.lib().goofy_gpu_batch_encode_noalloc(None, 3, None) == g.ERR_INVALID
    assert "NULL" in g.last_error()
    assert g.lib().goofy_gpu_batch_encode_noalloc(None, 0, None) == g.OK  # nothing to do
    items = _images(cuda, 4, 3)
    bad = _descs(items, "dst_a")
    bad[2] = (bad[2][0], bad[2][1], 6, 8, 64, 0)  # width % 4 != 0
    assert g.batch_encode_noalloc(bad) == g.ERR_WIDTH
    cuda.cuda.synchronize()
    assert all((it["dst_a"].cpu().numpy() == 0x11).all() for it in items)  # no image was encoded
