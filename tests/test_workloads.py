"""Synthetic workload generator: deterministic, and with the stated shapes."""
import hashlib

import numpy as np

from goofy_gb300 import workloads


def test_scene_deterministic_and_threads_agree(built, golden):
    a = workloads.scene(256, 256, 0)
    assert hashlib.sha256(a.tobytes()).hexdigest() == str(golden["cfg0_sha256"])
    b = workloads.scene(256, 256, 0, threads=4)
    np.testing.assert_array_equal(a, b)
    assert (a[:, 3::4] == 255).all()
    assert not np.array_equal(a, workloads.scene(256, 256, 1))


def test_scene_stride_padding(built):
    a = workloads.scene(64, 32, 3)
    b = workloads.scene(64, 32, 3, stride=64 * 4 + 48)
    np.testing.assert_array_equal(a, b[:, :256])


def test_stress_quarters(built):
    w = h = 256
    img = workloads.stress(w, h, 2).reshape(h, w, 4)
    q = w // 4
    blocks = lambda a: a.reshape(h // 4, 4, a.shape[1] // 4, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)
    const = blocks(img[:, q:2 * q])
    assert (const == const[:, :1]).all()               # one colour per block
    two = blocks(img[:, 2 * q:3 * q])
    assert max(len(np.unique(b.view(np.uint32))) for b in two) <= 2
    grey = img[:, 3 * q:]
    assert (grey[..., 0] == grey[..., 1]).all() and (grey[..., 1] == grey[..., 2]).all()
    assert len(np.unique(grey[..., 3])) > 200          # alpha is random
    assert len(np.unique(img[:, :q].reshape(-1))) == 256


def test_texture_batch_distribution(built):
    specs = [workloads.texture_spec(i) for i in range(1000)]
    ws = sorted({s[0] for s in specs})
    assert ws == [64, 128, 256, 512, 1024, 2048]
    mips = sum(s[2] for s in specs) / 1000
    etc = sum(s[3] for s in specs) / 1000
    assert 0.15 < mips < 0.25 and 0.45 < etc < 0.55
    chain = workloads.mip_chain(64, 256)
    assert chain[0] == (64, 256) and chain[-1] == (4, 4) and (4, 8) in chain
