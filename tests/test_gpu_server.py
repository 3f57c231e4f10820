"""Request server (continuous batching of host-memory requests): every
result equals the same request encoded alone, whatever mix it was served in,
in both data paths; the device budget delays admission instead of failing;
replay and the plain loop produce correct outputs and sane latencies."""
import numpy as np
import pytest

import goofy_gb300 as g
import oracle
from goofy_gb300 import workloads

pytestmark = pytest.mark.gpu


class Pinned:
    def __init__(self, nbytes):
        self.arr, self.ptr = g.pinned_array(nbytes)

    def free(self):
        g.host_free(self.ptr)


def make_requests(rng, n, pinned, max_side=1024):
    """Random sizes / codecs / strides; inputs from the scene generator."""
    reqs = []
    for i in range(n):
        w = int(4 << rng.integers(2, int(np.log2(max_side)) - 1))
        h = int(4 << rng.integers(2, int(np.log2(max_side)) - 1))
        if i % 5 == 2:
            w += 4 * int(rng.integers(1, 4))
        stride = 4 * w + [0, 16, 8][i % 3]
        img = np.zeros((h, stride), np.uint8)
        img[:, :4 * w] = workloads.scene(w, h, 500 + i)
        n_out = g.out_size(w, h)
        if pinned:
            src, dst = Pinned(img.size), Pinned(n_out)
            src.arr[:] = img.reshape(-1)
            dst.arr[:] = 0xEE
            src_arr, dst_arr = src.arr, dst.arr
        else:
            src, dst = None, None
            src_arr, dst_arr = img.reshape(-1), np.full(n_out, 0xEE, np.uint8)
        reqs.append(dict(w=w, h=h, stride=stride, codec=int(rng.integers(0, 2)), img=img, src=src_arr,
                         dst=dst_arr, bufs=(src, dst)))
    return reqs


def free_requests(reqs):
    for r in reqs:
        for b in r["bufs"]:
            if b is not None:
                b.free()


def alone(r):
    return oracle.encode(r["codec"], r["img"], r["w"], r["h"], stride=r["stride"])


@pytest.mark.parametrize("mode,pinned", [(g.SERVER_STAGED, False), (g.SERVER_STAGED, True), (g.SERVER_DIRECT, True)])
def test_results_equal_alone_and_in_the_mix(cuda, mode, pinned):
    rng = np.random.default_rng(11 + mode)
    reqs = make_requests(rng, 48, pinned)
    srv = g.Server(mode=mode, device_budget_bytes=64 << 20, max_batch_images=16, max_inflight_batches=3)
    try:
        tickets = []
        for r in reqs:  # all at once: they are served in mixed batches
            rc, t = srv.submit(r["codec"], r["dst"], r["src"], r["w"], r["h"], r["stride"])
            assert rc == g.OK, (rc, g.last_error())
            tickets.append(t)
        for r, t in zip(reqs, tickets):
            rc, times = srv.wait(t)
            assert rc == g.OK
            assert times.submit_ns <= times.admit_ns <= times.launch_ns <= times.done_ns
            np.testing.assert_array_equal(r["dst"], alone(r))
        st = srv.stats()
        assert st["requests_done"] == len(reqs) and st["launches"] < len(reqs)  # requests were batched
        assert st["max_batch"] > 1 and st["inflight_bytes"] == 0
        # the slowest launch's parts: enqueue and kernel within enqueue-to-completion, all read and reset
        assert 0 < st["max_kernel_ns"] and 0 < st["max_enqueue_ns"] < st["max_launch_ns"]
        assert 0 < st["slowest_kernel_ns"] <= st["slowest_gpu_span_ns"] and 0 < st["slowest_enqueue_ns"]
        assert st["slowest_enqueue_ns"] <= st["max_enqueue_ns"] and st["slowest_kernel_ns"] <= st["max_kernel_ns"]
        st = srv.stats()
        assert st["max_kernel_ns"] == st["max_enqueue_ns"] == st["max_launch_ns"] == 0
        assert st["slowest_kernel_ns"] == st["slowest_gpu_span_ns"] == st["slowest_enqueue_ns"] == 0
        # the same request served on its own gives the same bytes
        r = reqs[5]
        r["dst"][:] = 0
        rc, t = srv.submit(r["codec"], r["dst"], r["src"], r["w"], r["h"], r["stride"])
        assert rc == g.OK and srv.wait(t)[0] == g.OK
        np.testing.assert_array_equal(r["dst"], alone(r))
    finally:
        srv.close()
        free_requests(reqs)


def test_budget_delays_admission(cuda):
    """A budget that holds only a couple of requests: everything still
    completes, in order of admission, and over-budget requests are refused."""
    rng = np.random.default_rng(5)
    reqs = make_requests(rng, 24, True, max_side=512)
    biggest = max(r["stride"] * r["h"] + g.out_size(r["w"], r["h"]) for r in reqs)
    srv = g.Server(mode=g.SERVER_STAGED, device_budget_bytes=max(2 * biggest + (1 << 16), 1 << 20),
                   max_batch_images=8, max_inflight_batches=2)
    try:
        tickets = [srv.submit(r["codec"], r["dst"], r["src"], r["w"], r["h"], r["stride"])[1] for r in reqs]
        admits = []
        for r, t in zip(reqs, tickets):
            rc, times = srv.wait(t)
            assert rc == g.OK
            admits.append(times.admit_ns)
            np.testing.assert_array_equal(r["dst"], alone(r))
        assert admits == sorted(admits)
        huge = np.zeros(16, np.uint8)
        rc, _ = srv.submit(0, huge, huge, 4096, 4096, 16384)
        assert rc == g.ERR_TOO_LARGE
    finally:
        srv.close()
        free_requests(reqs)


def test_ticket_ring_and_argument_checks(cuda):
    rng = np.random.default_rng(9)
    reqs = make_requests(rng, 1, True, max_side=64)
    r = reqs[0]
    srv = g.Server(mode=g.SERVER_DIRECT, max_requests=16)
    try:
        got = [srv.submit(r["codec"], r["dst"], r["src"], r["w"], r["h"], r["stride"]) for _ in range(17)]
        assert all(rc == g.OK for rc, _ in got[:16]) and got[16][0] == g.ERR_BUSY
        for rc, t in got[:16]:
            assert srv.wait(t)[0] == g.OK
        assert srv.wait(got[0][1])[0] == g.ERR_INVALID  # already released
        assert srv.submit(r["codec"], r["dst"], r["src"], 6, 8, 64)[0] == g.ERR_WIDTH
        assert srv.submit(7, r["dst"], r["src"], 8, 8, 64)[0] == g.ERR_INVALID
        np.testing.assert_array_equal(r["dst"], alone(r))
    finally:
        srv.close()
        free_requests(reqs)


@pytest.mark.parametrize("completion", [g.COMPLETION_CALLBACK, g.COMPLETION_EVENT])
@pytest.mark.parametrize("mode", [g.SERVER_STAGED, g.SERVER_DIRECT])
def test_replay_and_plain_loop(cuda, mode, completion):
    """Open-loop replay through the server (a launch's completion seen by a
    host callback, or by the server's thread waiting on its last event) and through the plain
    loop: every request's blocks equal its encode alone."""
    rng = np.random.default_rng(21)
    reqs = make_requests(rng, 64, True, max_side=512)
    arr = g.requests_array([(r["src"], r["dst"], r["w"], r["h"], r["stride"], r["codec"]) for r in reqs])
    arrival = np.cumsum(rng.exponential(20e3, len(reqs))).astype(np.int64)  # ~50k requests/s
    srv = g.Server(mode=mode, completion=completion)
    try:
        rc, lat, wall, stamps = srv.replay(arr, arrival, with_times=True)
        assert rc == g.OK and (lat > 0).all() and wall > 0
        # submit <= admit <= launch <= done for every request, done - latency = its scheduled arrival
        assert (np.diff(stamps, axis=1) >= 0).all()
        sched = stamps[:, 3] - lat
        np.testing.assert_array_equal(np.diff(sched), np.diff(arrival))
        for r in reqs:
            np.testing.assert_array_equal(r["dst"], alone(r))
            r["dst"][:] = 0
        rc, lat, wall = g.plain_replay(arr, arrival)
        assert rc == g.OK and (lat > 0).all()
        for r in reqs:
            np.testing.assert_array_equal(r["dst"], alone(r))
    finally:
        srv.close()
        free_requests(reqs)


@pytest.mark.parametrize("mode", [g.SERVER_STAGED, g.SERVER_DIRECT])
def test_quality_reports_each_requests_psnr(cuda, mode):
    """With quality on, every request's RGB PSNR (measured on the GPU from the
    batch's own blocks, in the same launches) equals the harness's figure for
    that request alone: decode with the harness's decoder, getMsePsnr."""
    rng = np.random.default_rng(33)
    reqs = make_requests(rng, 40, True, max_side=512)
    srv = g.Server(mode=mode, quality=True)
    try:
        tickets = [srv.submit(r["codec"], r["dst"], r["src"], r["w"], r["h"], r["stride"]) for r in reqs]
        assert all(rc == g.OK for rc, _ in tickets)
        for r, (_, tk) in zip(reqs, tickets):
            rc, tm = srv.wait(tk)
            assert rc == g.OK
            blocks = alone(r)
            np.testing.assert_array_equal(r["dst"], blocks)
            dec, bad = oracle.decode(r["codec"], blocks, r["w"], r["h"])
            src = np.ascontiguousarray(r["img"][:, :4 * r["w"]])
            assert bad == 0
            assert tm.psnr_rgb == oracle.psnr_rgb(oracle.sq_error(src, dec, r["w"], r["h"]), r["w"], r["h"])
    finally:
        srv.close()
        free_requests(reqs)
    # without quality the field stays 0
    reqs = make_requests(rng, 4, True, max_side=64)
    srv = g.Server(mode=mode)
    try:
        for r in reqs:
            rc, tk = srv.submit(r["codec"], r["dst"], r["src"], r["w"], r["h"], r["stride"])
            assert rc == g.OK and srv.wait(tk)[1].psnr_rgb == 0.0
    finally:
        srv.close()
        free_requests(reqs)
