"""GPU decoder and the encode-quality reduction against the oracle (which is
pinned to the reference's own decoder and PSNR): decoded pixels bit-exact,
squared-error sums exact, RGB PSNR identical."""
import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu


def _etc1_blocks(rng, n):
    blocks = rng.integers(0, 256, (n, 8), dtype=np.uint8)
    for b in blocks:
        if b[3] & 2:
            for c in range(3):
                base, d = int(b[c]) >> 3, int(b[c]) & 7
                d = d - 8 if d >= 4 else d
                if not 0 <= base + d <= 31:
                    b[c] = base << 3
    return blocks


def _gpu_decode(torch, codec, blocks, w, h):
    d_blocks = torch.from_numpy(np.ascontiguousarray(blocks).reshape(-1)).cuda()
    rgba = torch.full((h * 4 * w,), 0x77, dtype=torch.uint8, device="cuda")
    bad = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = g.decode_device(codec, rgba, 4 * w, d_blocks, w, h, bad, torch.cuda.current_stream().cuda_stream)
    assert rc == g.OK, (rc, g.last_error())
    torch.cuda.synchronize()
    return rgba.cpu().numpy().reshape(h, 4 * w), int(bad.item())


@pytest.mark.parametrize("codec", [0, 1])
def test_decode_random_and_encoded_blocks(cuda, golden, codec):
    rng = np.random.default_rng(3 + codec)
    w, h = 256, 64
    random = rng.integers(0, 256, (w * h // 16, 8), dtype=np.uint8) if codec == 0 else _etc1_blocks(rng, w * h // 16)
    encoded = golden["kat_bc1" if codec == 0 else "kat_etc1s"]
    kw, kh = int(golden["kat_width"]), int(golden["kat_height"])
    for blocks, bw_, bh_ in ((random, w, h), (encoded, kw, kh)):
        got, bad = _gpu_decode(cuda, codec, blocks, bw_, bh_)
        want, wbad = oracle.decode(codec, blocks, bw_, bh_)
        assert bad == wbad == 0
        np.testing.assert_array_equal(got, want)


def test_decode_counts_etc2_mode_blocks(cuda):
    blk = np.zeros((16, 8), np.uint8)
    blk[:, 0] = (31 << 3) | 3   # R 31 + delta +3 -> out of range: an ETC2 mode
    blk[:, 3] = 2               # differential
    got, bad = _gpu_decode(cuda, 1, blk, 16, 16)
    want, wbad = oracle.decode(1, blk, 16, 16)
    assert bad == wbad == 16
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("codec", [0, 1])
def test_error_sums_and_psnr(cuda, codec):
    for (w, h, img) in ((256, 256, workloads.scene(256, 256, 0)), (1028, 36, workloads.scene(1028, 36, 4)),
                        (4096, 4096, workloads.stress(4096, 4096, 2))):
        blocks = oracle.encode(codec, img, w, h, threads=0)
        dec, _ = oracle.decode(codec, blocks, w, h)
        want = oracle.sq_error(img, dec, w, h)
        d_img = cuda.from_numpy(np.ascontiguousarray(img).reshape(-1)).cuda()
        d_blk = cuda.from_numpy(blocks).cuda()
        rc, psnr, sums = g.psnr_rgb(codec, d_blk, d_img, w, h, 4 * w)
        assert rc == g.OK, g.last_error()
        np.testing.assert_array_equal(sums[:4], want)
        assert sums[4] == 0
        assert psnr == oracle.psnr_rgb(want, w, h)


def test_error_sums_unaligned_source(cuda):
    w, h = 72, 24
    img = workloads.scene(w, h, 11)
    blocks = oracle.encode(1, img, w, h)
    dec, _ = oracle.decode(1, blocks, w, h)
    want = oracle.sq_error(img, dec, w, h)
    stride = 4 * w + 4
    buf = np.zeros(h * stride + 8, np.uint8)
    buf[4:4 + h * stride].reshape(h, stride)[:, :4 * w] = img
    d_buf = cuda.from_numpy(buf).cuda()
    d_blk = cuda.from_numpy(blocks).cuda()
    sums = cuda.zeros(6, dtype=cuda.int64, device="cuda")
    assert g.block_error_device(1, d_blk, d_buf.data_ptr() + 4, w, h, stride, sums) == g.OK
    cuda.cuda.synchronize()
    np.testing.assert_array_equal(sums.cpu().numpy()[:4].astype(np.uint64), want)


@pytest.mark.parametrize("codec", [0, 1])
def test_full_mse_psnr_record(cuda, codec):
    """The harness's whole getMsePsnr record (per channel, max / min, RGB,
    luminosity) measured on the GPU equals the oracle's restatement, which
    does the harness's own double arithmetic; random alpha makes mse_a non-zero."""
    rng = np.random.default_rng(3 + codec)
    for (w, h) in ((256, 256), (1028, 36), (2048, 1024)):
        img = workloads.scene(w, h, w + codec)
        img.reshape(h, w, 4)[..., 3] = rng.integers(0, 256, (h, w))
        blocks = oracle.encode(codec, img, w, h, threads=0)
        dec, _ = oracle.decode(codec, blocks, w, h)
        want = oracle.mse_psnr(img, dec, w, h)
        q = g.mse_psnr(codec, cuda.from_numpy(blocks).cuda(), cuda.from_numpy(np.ascontiguousarray(img).reshape(-1)).cuda(),
                       w, h, 4 * w)
        assert q["unsupported_blocks"] == 0
        for k, v in want.items():
            if k.endswith("_y"):  # exact integers vs the harness's rounded 0.21 / 0.72 / 0.07 products
                assert q[k] == pytest.approx(v, rel=1e-10), k
            else:
                assert q[k] == v, k
