"""bench.py's host-side bookkeeping on CPU: the clock record taken during the
timed region, the committed per-launch DRAM traffic the roofline quotes, and
the peak it is measured against."""
import json
import os

import bench

ROW = "0, {sm}, 2070, 900.0, 0x0, {hw}, Not Active, Not Active, {cap}, 3996, 3996"


def _summary(lines):
    c = bench.ClockSampler(0)
    c.lines = lines
    return c.summary()


def test_clock_summary_median_reasons_and_memory_clock():
    s = _summary([ROW.format(sm=2070, hw="Not Active", cap="Not Active"),
                  ROW.format(sm=1980, hw="Not Active", cap="Active"),
                  ROW.format(sm=2070, hw="Not Active", cap="Not Active")])
    assert s["sm_mhz"] == 2070 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    assert s["mem_mhz"] == 3996 and s["mem_max_mhz"] == 3996 and s["power_w"] == 900.0
    assert _summary([ROW.format(sm=1500, hw="Active", cap="Not Active")])["reasons"] == ["hw_slowdown"]


def test_clock_summary_without_samples_or_memory_fields():
    assert _summary([])["samples"] == 0
    short = "0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active"
    s = _summary([short, "garbage", ""])
    assert s["samples"] == 1 and "mem_mhz" not in s


def test_roofline_traffic_comes_from_the_committed_profiles():
    """Every kernel the roofline can name has its ncu read + write bytes in
    profiles/, and they are close to the algorithmic 4.5 B/px of a launch
    (less where L2 still holds part of the output at the end)."""
    algorithmic = 4.5 * 8192 * 8192
    for key in ("encode_image_tma_bc1_8192", "encode_image_tma_etc1s_8192"):
        t = bench.read_traffic(key)
        assert t is not None, key
        assert 0.9 * algorithmic < t <= 1.02 * algorithmic, (key, t)
    assert bench.read_traffic("no_such_kernel") is None


def test_dropin_latency_calls_each_entry_point_on_contiguous_corners():
    """The drop-in timing passes each entry point a contiguous copy of the
    image's top-left side x side corner with the drop-in's own arguments."""
    import numpy as np

    seen = []

    class FakeLib:
        def out_size(self, w, h):
            return w * h // 2

        def _call(self, name, out, src, w, h, stride):
            assert src.flags.c_contiguous and src.shape == (h, 4 * w) and stride == 4 * w
            assert out.size == w * h // 2 and src[0, 0] == 7
            seen.append((name, w))
            return 0

        def compressDXT1(self, *a):
            return self._call("bc1", *a)

        def compressETC1(self, *a):
            return self._call("etc1s", *a)

        def last_error(self):
            return ""

    img = np.full((512, 2048), 7, np.uint8)
    res = bench.run_dropin_latency(FakeLib(), img, sides=(64, 512), calls=4)
    assert set(res) == {"64x64", "512x512", "note"}
    assert all(set(res[k]) == {"bc1", "etc1s"} and min(res[k].values()) >= 0 for k in ("64x64", "512x512"))
    assert len(seen) == 2 * 2 * (5 + 4) and {s for _, s in seen} == {64, 512}


def test_peak_is_the_measured_copy_bandwidth():
    peak, kind = bench.read_peaks()
    path = os.path.join(bench.ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        assert kind == "measured" and peak == float(json.load(open(path))["hbm_gbs"])
    else:
        assert (peak, kind) == (6800.0, "fallback")


class _FakeTensor:
    count = [0]

    def __init__(self, n):
        self.n = n
        _FakeTensor.count[0] += 1
        self.ptr = 4096 * _FakeTensor.count[0]

    def fill_(self, v):
        return self

    def to(self, device):
        return _FakeTensor(self.n)

    def reshape(self, *a):
        return self

    def data_ptr(self):
        return self.ptr


class _FakeEvent:
    clock = [0.0]

    def __init__(self, enable_timing=False):
        self.t = None

    def record(self, stream):
        _FakeEvent.clock[0] += 0.005  # 5 us between consecutive records
        self.t = _FakeEvent.clock[0]

    def synchronize(self):
        pass

    def elapsed_time(self, other):
        return other.t - self.t


class _FakeTorch:
    uint8 = "u8"

    class cuda:
        Event = _FakeEvent

    @staticmethod
    def empty(n, dtype=None, device=None):
        return _FakeTensor(n)

    @staticmethod
    def from_numpy(a):
        return _FakeTensor(a.size)


def test_small_configs_bookkeeping():
    """run_small_configs: the stress image's launches run back to back between
    two events with the input rotating over 4 copies and the output over 4
    buffers; the 256x256 latency brackets each launch alone after a flush."""
    import types

    import numpy as np

    calls = []

    class FakeLib:
        OK, CODEC_BC1, CODEC_ETC1S = 0, 0, 1

        def out_size(self, w, h):
            return w * h // 2

        def compress_device(self, c, dst, src, w, h, stride, sh):
            calls.append((c, dst, src, w, stride))
            return 0

        def status_string(self, rc):
            return "?"

        def last_error(self):
            return ""

    work = types.SimpleNamespace(scene=lambda w, h, s: np.zeros((h, 4 * w), np.uint8),
                                 stress=lambda w, h, s: np.zeros((h, 4 * w), np.uint8))
    stream = types.SimpleNamespace(cuda_stream=0, device="cuda:0")
    args = types.SimpleNamespace(steps=10)
    res = bench.run_small_configs(args, FakeLib(), _FakeTorch, work, (0, 1), stream, peak=6800.0)
    n = 40  # max(steps, 40) launches a round
    big = [c for c in calls if c[3] == 4096]
    small = [c for c in calls if c[3] == 256]
    assert len(big) == 2 * (2 + 3 * n) + (2 + 3 * n) and {s for *_, s in big} == {16384}
    assert len({c[2] for c in big}) == 4 and len({c[1] for c in big}) == 4  # 4 inputs, 4 outputs
    assert len(small) == 2 * (62 + 2 + 3 * 200) and {s for *_, s in small} == {1024}
    r = res["4096x4096"]["etc1s"]
    assert r["mean_launch_us"] == round(5.0 / n, 2)  # one 5 us tick of the fake clock over n launches
    assert r["frac"] == round(4.5 * 4096 * 4096 / (5.0 / n) / 1e3 / 6800.0, 4)
    assert res["256x256"]["bc1"]["latency_us"] == 5.0
    assert res["4096x4096"]["alternating_pair_us"] == round(2 * 5.0 / n, 2)


def test_summary_reads_the_sections_it_quotes():
    line = {"ms_per_step": 0.1, "config": {"pixels_per_step": 2 * 8192 * 8192},
            "per_codec": {"bc1": {"mean_launch_us": 43.0}, "etc1s": {"mean_launch_us": 46.0}},
            "roofline": {"frac": 0.95}, "small_configs": {"4096x4096": {"bc1": {"mean_launch_us": 14.0,
                                                                                 "frac": 0.8}}},
            "serving": {"staged": {"loads": {"50%": {"p99_ms": 0.5, "by_class": {"probe_1024x1024":
                                                                               {"p99_ms": 0.6}}}}}}}
    s = bench.summary(line, 6800.0)
    assert s["step_us"] == 100.0 and s["bc1_8192_us"] == 43.0 and s["stress4096_bc1_frac"] == 0.8
    assert s["stress4096_etc1s_us"] is None and s["serve_staged_50pct_probe_p99_ms"] == 0.6
    assert s["step_frac"] == round(4.5 * 2 * 8192 * 8192 / 1e-4 / 1e9 / 6800.0, 4)
    assert len(json.dumps(s)) < 1000
