"""Benchmark: Goofy BC1 + ETC1s encode on GB300, one JSON line on stdout.

Workload (one step): encode one 8192x8192 RGBA8 scene (stride 32768 B,
seed 1, noise periods x32, 2048 rectangles) with BC1 and with ETC1s -- two
kernel launches, 2 x 67,108,864 pixels.  Two device copies of the image
alternate between the codecs, so every launch reads 256 MiB that the
previous launch did not touch (inputs larger than the 129 MB L2).

* value      -- MPix/s with inputs resident in HBM (device-pointer C ABI),
                CUDA events around K steps on the launching stream.
* e2e        -- the same metric through the host C ABI
                (goofy_gpu_compress_host, the engine under goofy::compress*)
                from pinned host memory, copies in and out inside the region.
* roofline   -- dominant kernel: 4.5 algorithmic B/px (4 read + 0.5 written)
                x pixels per launch / its mean launch duration (K launches
                back to back between two CUDA events, right after the timed
                steps, inputs and outputs alternating between two buffers
                each), against the measured HBM copy bandwidth.  No event
                is recorded between two launches of a timed loop: one there
                delays the next launch's start by a few microseconds.
* cpu_baseline -- the oracle port timed on this host's cores (bounded sample).
* both_codecs_one_pass -- beside the headline: the same two outputs from one
                read of the image (goofy_gpu_compress_both_*), device and host.
* small_configs -- the 4096x4096 stress image (launches back to back over
                inputs rotating through 256 MiB) and the 256x256 scene
                (latency of one launch with L2 cold).
* summary    -- the figures above that the other sections explain, in one
                short object at the end of the line.

``--impl reference`` times the reference's CPU implementation of the path on
this host's cores instead (the reference compiled from its own sources where
they exist, else the oracle port of it), with every host thread.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DXT1/ETC1s MPix/s on 1 GB300 vs HBM roofline, batched vs plain; p50/p99 latency"
W = H = 8192
SEED, PERIOD_SCALE, RECTS = 1, 32, 2048
ALG_BYTES_PER_PX = 4.5
WORKLOAD = ("plain BC1 + ETC1s encode of one 8192x8192 RGBA8 synthetic scene (stride 32768 B, seed 1, "
            "value-noise periods x32, 2048 rectangles)")
# the same `config` on both arms (GPU and reference CPU)
CONFIG = {"workload": WORKLOAD, "pixels_per_step": 2 * W * H,
          "l2": "inputs larger than L2: 256 MiB per image (the GPU's L2 is 129 MB); the GPU arm alternates two "
                "device copies of it between the codecs"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--soak-s", type=float, default=1.5, help="seconds of the same loop before the timed region "
                                                             "while clocks are sampled")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--serve-seconds", type=float, default=4.0, help="length of each offered-load run")
    p.add_argument("--serve-soak-s", type=float, default=30.0, help="length of the staged server's 10%% load soak "
                                                                     "window (0: none)")
    p.add_argument("--batch-textures", type=int, default=1000)
    p.add_argument("--sweep", action="store_true", help="print every tile shape's launch time to stderr")
    p.add_argument("--profile", choices=["encode", "quality", "mips", "batch", "batch-pipeline", "both"],
                   help="only run a few launches of one kernel family (for ncu captures) and exit")
    p.add_argument("--profile-size", default="4096", help="image size for --profile: a side (square) or WxH")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world):
    """The slowest rank's figure (a replica job ends when its last GPU ends);
    CPU tensors over the gloo group, no data-path collective."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate_mpix_s(world, px_per_rank_step, steps, slowest_ms):
    """Whole-job throughput: every rank's pixels over the slowest rank's time."""
    return world * px_per_rank_step * steps / (slowest_ms / 1e3) / 1e6


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_traffic(kernel_key):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/*.md, a line `traffic <kernel_key> <bytes>`), or None."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for name in sorted(os.listdir(pdir)):
        if not name.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(pdir, name)):
            parts = line.strip().strip("`").split()
            if len(parts) == 3 and parts[0] == "traffic" and parts[1] == kernel_key:
                try:
                    return int(parts[2])
                except ValueError:
                    pass
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,clocks.mem,clocks.max.mem")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, mem, mem_mx, power, reasons = [], [], [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
            try:  # memory clock and power: reported beside the SM clock, not used to accept a run
                power.append(float(f[3]))
                mem.append(float(f[9]))
                mem_mx.append(float(f[10]))
            except (ValueError, IndexError):
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
               "samples": len(sm)}
        if mem:
            out.update(mem_mhz=statistics.median(mem), mem_max_mhz=max(mem_mx), power_w=statistics.median(power))
        return out


def cpu_throttle_stats():
    """CPU-quota throttling of this process's cgroup so far (cgroup v2
    cpu.stat, else v1 cpu/cpu.stat): periods, throttled periods and
    throttled microseconds; {} where the files are absent."""
    for path, unit in (("/sys/fs/cgroup/cpu.stat", 1.0), ("/sys/fs/cgroup/cpu/cpu.stat", 1e-3),
                       ("/sys/fs/cgroup/cpu,cpuacct/cpu.stat", 1e-3)):
        try:
            kv = dict(l.split() for l in open(path) if len(l.split()) == 2)
        except OSError:
            continue
        us = kv.get("throttled_usec")
        us = float(us) if us is not None else float(kv.get("throttled_time", 0)) * unit
        return {"periods": int(kv.get("nr_periods", 0)), "throttled": int(kv.get("nr_throttled", 0)),
                "throttled_us": us}
    return {}


def pressure_totals():
    """Host pressure stall information (/proc/pressure): microseconds in
    which some task waited for CPU, memory or IO, so far; {} if absent."""
    out = {}
    for res in ("cpu", "memory", "io"):
        try:
            for line in open("/proc/pressure/" + res):
                if line.startswith("some"):
                    out[res] = int(line.split("total=")[1])
        except (OSError, IndexError, ValueError):
            pass
    return out


def window_diagnostics(thr0, psi0, thr1, psi1, st):
    """Per serving window: CPU-quota throttling, host pressure stall time and
    the slowest launch's parts (server stats read and reset around the window)."""
    return {"cpu_quota_throttling": throttle_delta(thr0, thr1),
            "host_pressure_stall_ms": {k: round((psi1[k] - psi0[k]) / 1e3, 3) for k in psi1 if k in psi0},
            "launch_max_ms": {"enqueue": round(st["max_enqueue_ns"] / 1e6, 3),
                              "kernel": round(st["max_kernel_ns"] / 1e6, 3),
                              "enqueue_to_done": round(st["max_launch_ns"] / 1e6, 3)},
            "slowest_launch_ms": {"enqueue_to_done": round(st["max_launch_ns"] / 1e6, 3),
                                  "enqueue": round(st["slowest_enqueue_ns"] / 1e6, 3),
                                  "gpu_first_to_last_op": round(st["slowest_gpu_span_ns"] / 1e6, 3),
                                  "kernel": round(st["slowest_kernel_ns"] / 1e6, 3)}}


def throttle_delta(a, b):
    if not a or not b:
        return None
    return {k: round(b[k] - a[k], 1) for k in a}


def cpu_quota():
    """The cgroup's CPU quota as "quota period" (v2 cpu.max / v1 cfs files), or None."""
    try:
        return open("/sys/fs/cgroup/cpu.max").read().strip()
    except OSError:
        pass
    try:
        q = open("/sys/fs/cgroup/cpu/cpu.cfs_quota_us").read().strip()
        p = open("/sys/fs/cgroup/cpu/cpu.cfs_period_us").read().strip()
        return "%s %s" % (q, p)
    except OSError:
        return None


def cpu_encode_all(lib_fn, img, threads, outs=None):
    """Both codecs over the whole image; returns seconds."""
    import numpy as np

    if outs is None:
        outs = [np.empty((W // 4) * (H // 4) * 8, np.uint8) for _ in range(2)]
    t0 = time.perf_counter()
    for codec in (0, 1):
        rc = lib_fn(codec, outs[codec].ctypes.data, img.ctypes.data, W, H, 4 * W, threads)
        assert rc > 0, rc
    return time.perf_counter() - t0


def cpu_model():
    """The host CPU's model name (lscpu / /proc/cpuinfo), for the baseline's label."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.machine()


def cpu_baseline(img, gpu_outputs, budget_s=12.0):
    """The reference's own CPU encoder (its SSE2 path on x86-64, its scalar
    path elsewhere; the oracle port only where neither was built) on this
    host's cores: all threads, best of a few full-image passes of both codecs.
    The CPU outputs of the last pass double as the check of the GPU outputs."""
    import numpy as np

    import oracle

    fn, kind, label = oracle.ref_encoder()
    cores = os.cpu_count() or 1
    times = []
    outs = [np.empty((W // 4) * (H // 4) * 8, np.uint8) for _ in range(2)]
    t_start = time.perf_counter()
    while len(times) < 3 or (time.perf_counter() - t_start < budget_s / 2 and len(times) < 20):
        times.append(cpu_encode_all(fn, img, cores, outs))
        if time.perf_counter() - t_start > budget_s:
            break
    best = min(times)
    t1 = cpu_encode_all(fn, img, 1)
    px = 2 * W * H
    return {"value": round(px / best / 1e6, 1), "unit": "MPix/s", "cores": cores, "kind": kind,
            "sample": "full 8192x8192 image, BC1 + ETC1s, best of %d passes, block rows striped over %d threads"
                      % (len(times), cores),
            "single_thread_mpix_s": round(px / t1 / 1e6, 1),
            "median_mpix_s": round(px / statistics.median(times) / 1e6, 1),
            "implementation": label, "cpu": "%s, %s" % (cpu_model(), platform.machine()),
            "gpu_output_bit_exact": bool(all(np.array_equal(outs[c], gpu_outputs[c]) for c in (0, 1)))}


def run_dropin_latency(g, img, sides=(256, 1024, 4096), calls=50):
    """Wall time of one goofy::compressDXT1 / compressETC1 call (the drop-in
    entry points, synchronous, host buffers) as a caller of the reference sees
    it: contiguous numpy (pageable) copies of the scene's top-left corner,
    median of `calls` calls after five untimed ones."""
    import numpy as np

    res = {}
    for side in sides:
        src = np.ascontiguousarray(img[:side, :4 * side])
        out = np.empty(g.out_size(side, side), np.uint8)
        row = {}
        for name, fn in (("bc1", g.compressDXT1), ("etc1s", g.compressETC1)):
            for _ in range(5):
                if fn(out, src, side, side, 4 * side) != 0:
                    raise RuntimeError(g.last_error())
            ts = []
            for _ in range(calls):
                t0 = time.perf_counter()
                fn(out, src, side, side, 4 * side)
                ts.append(time.perf_counter() - t0)
            row[name] = round(1e6 * statistics.median(ts), 1)
        res["%dx%d" % (side, side)] = row
    res["note"] = ("median wall time of one drop-in call from Python (ctypes) with pageable numpy buffers, "
                   "%d calls per entry; it includes a kernel launch and a stream synchronisation" % calls)
    return res


def summary(line, peak):
    """The figures of the line in one short flat object (the line's last key)."""
    def get(*path):
        d = line
        for k in path:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    out = {"step_us": round(1e3 * line["ms_per_step"], 2),
           "bc1_8192_us": get("per_codec", "bc1", "mean_launch_us"),
           "etc1s_8192_us": get("per_codec", "etc1s", "mean_launch_us"),
           "step_frac": round(ALG_BYTES_PER_PX * line["config"]["pixels_per_step"] / (line["ms_per_step"] * 1e-3)
                              / 1e9 / peak, 4),
           "dominant_frac": get("roofline", "frac"),
           "tiles": get("tiles"), "cached_tiles_step_ratio": get("tile_cache", "cached_over_tuned"),
           "stress4096_bc1_us": get("small_configs", "4096x4096", "bc1", "mean_launch_us"),
           "stress4096_etc1s_us": get("small_configs", "4096x4096", "etc1s", "mean_launch_us"),
           "stress4096_bc1_frac": get("small_configs", "4096x4096", "bc1", "frac"),
           "stress4096_etc1s_frac": get("small_configs", "4096x4096", "etc1s", "frac"),
           "scene256_latency_us": [get("small_configs", "256x256", c, "latency_us") for c in ("bc1", "etc1s")],
           "both_one_pass_us": get("both_codecs_one_pass", "mean_launch_us"),
           "batched_speedup_vs_plain": get("batched", "speedup_vs_plain"),
           "batch_16x2048_us": get("batch_16x2048", "mean_call_us"), "batch_16x2048_frac": get("batch_16x2048", "frac"),
           "batched_mpix_s": get("batched", "batched_mpix_s"),
           "e2e_mpix_s": get("e2e", "value"),
           "cpu_mpix_s": get("cpu_baseline", "value"), "cpu_kind": get("cpu_baseline", "kind")}
    for mode in ("staged", "direct"):
        l50 = get("serving", mode, "loads", "50%")
        if l50:
            out["serve_%s_50pct_p99_ms" % mode] = l50["p99_ms"]
            out["serve_%s_50pct_probe_p99_ms" % mode] = get("serving", mode, "loads", "50%", "by_class",
                                                            "probe_1024x1024", "p99_ms")
    out["serve_vs_plain"] = get("serving", "plain", "server_vs_plain")
    out["serve_staged_soak_10pct_max_ms"] = get("serving", "staged", "soak_10pct", "max_ms")
    return out


def back_to_back_us(torch, stream, launch, n, rounds=3):
    """Mean duration of one launch: `n` launches back to back between two CUDA
    events on `stream` (no event between two launches), median of `rounds`
    rounds after two untimed launches.  launch(k) enqueues launch k."""
    for k in range(2):
        launch(k)
    ts = []
    for _ in range(rounds):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(n):
            launch(k)
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e3 / n)
    return statistics.median(ts)


def run_small_configs(args, g, torch, workloads, codecs, stream, peak):
    """The two other single-image workloads.

    * 4096x4096 stress quarters (seed 2): each codec as launches back to back
      between two CUDA events, the input rotating over 4 device copies of the
      64 MiB image (256 MiB, twice the L2) and the output over 4 buffers, so
      no launch finds its input in L2.  Mean launch time and the fraction of
      the measured HBM peak at 4.5 B/px.  Also the alternating BC1 / ETC1s
      pair, as a caller encoding the image with both codecs issues it.
    * 256x256 scene (seed 0): the latency of one launch (timed alone between
      its own events after a 256 MiB write empties L2, mean of 60) and the
      mean launch time back to back (its 256 KiB input stays in L2)."""
    sh = stream.cuda_stream
    dev = stream.device
    side = 4096
    img = workloads.stress(side, side, 2)
    n_out = g.out_size(side, side)
    srcs = [torch.from_numpy(img.reshape(-1)).to(dev) for _ in range(4)]
    outs = [torch.empty(n_out, dtype=torch.uint8, device=dev) for _ in range(4)]
    n = max(args.steps, 40)
    names = {g.CODEC_BC1: "bc1", g.CODEC_ETC1S: "etc1s"}
    stress = {"workload": "4096x4096 stress quarters (seed 2: uniform noise, constant blocks, two-colour blocks, "
                          "grey with random alpha)"}

    def check(rc):
        if rc != g.OK:
            raise RuntimeError("stress: %s %s" % (g.status_string(rc), g.last_error()))

    for c in codecs:
        us = back_to_back_us(torch, stream, lambda k, c=c: check(
            g.compress_device(c, outs[k % 4].data_ptr(), srcs[(k + 1) % 4].data_ptr(), side, side, 4 * side, sh)), n)
        gbs = ALG_BYTES_PER_PX * side * side / us / 1e3
        stress[names[c]] = {"mean_launch_us": round(us, 2), "mpix_s": round(side * side / us, 1),
                            "hbm_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
    pair_us = back_to_back_us(torch, stream, lambda k: check(
        g.compress_device(codecs[k % 2], outs[k % 4].data_ptr(), srcs[(k + 1) % 4].data_ptr(), side, side, 4 * side,
                          sh)), 2 * (n // 2)) * 2
    stress["alternating_pair_us"] = round(pair_us, 2)
    stress["timing"] = ("mean of %d launches back to back between two CUDA events (median of 3 rounds), input "
                        "rotating over 4 device copies (256 MiB > L2), output over 4 buffers; alternating_pair_us = "
                        "one BC1 launch + one ETC1s launch, alternating" % n)
    del srcs, outs

    side = 256
    img = workloads.scene(side, side, 0)
    src = torch.from_numpy(img.reshape(-1)).to(dev)
    dst = [torch.empty(g.out_size(side, side), dtype=torch.uint8, device=dev) for _ in range(2)]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    small = {"workload": "256x256 scene (seed 0, stride 1024 B)"}
    for c in codecs:
        ts = []
        for r in range(62):
            flush.fill_(r & 0xff)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rc = g.compress_device(c, dst[0].data_ptr(), src.data_ptr(), side, side, 4 * side, sh)
            e1.record(stream)
            check(rc)
            e1.synchronize()
            if r >= 2:
                ts.append(e0.elapsed_time(e1) * 1e3)
        b2b = back_to_back_us(torch, stream, lambda k, c=c: check(
            g.compress_device(c, dst[k % 2].data_ptr(), src.data_ptr(), side, side, 4 * side, sh)), 200)
        small[names[c]] = {"latency_us": round(statistics.mean(ts), 2), "latency_median_us": round(statistics.median(ts), 2),
                           "latency_min_us": round(min(ts), 2), "back_to_back_us": round(b2b, 2)}
    small["timing"] = ("latency: one launch between its own two CUDA events after a 256 MiB write (L2 cold), mean of "
                       "60; such an event pair reads in steps of about 2 us on this GPU, the same step in every repeat, "
                       "so this is an upper bound at that resolution; back_to_back: mean of 200 launches between two "
                       "events (input L2-resident)")
    del flush
    return {"4096x4096": stress, "256x256": small}


def run_batch_16x2048(args, g, torch, workloads, stream, device):
    """16 textures of 2048x2048 (8 BC1, 8 ETC1s; 256 MiB of input, twice the
    L2) in one call of the pipelined batch kernel, its descriptors passed as
    the kernel's parameter: mean of launches back to back between two
    events, outputs alternating between two sets."""
    side, n = 2048, 16
    img = workloads.scene(side, side, 3, threads=0)
    srcs = [torch.from_numpy(img.reshape(-1)).to(stream.device) for _ in range(n)]
    outs = [[torch.empty(g.out_size(side, side), dtype=torch.uint8, device=stream.device) for _ in range(n)]
            for _ in range(2)]
    arrs = [g.images_array([(srcs[i].data_ptr(), outs[k][i].data_ptr(), side, side, 4 * side, i % 2)
                            for i in range(n)]) for k in range(2)]
    b = g.Batch(n, device)
    try:
        assert b.set_tile(512, 2, 1024, 1) == g.OK
        sh = stream.cuda_stream
        us = back_to_back_us(torch, stream, lambda k: b.encode(arrs[k % 2], sh), max(args.steps, 20))
        same = all(bool(torch.equal(outs[0][i], outs[1][i])) for i in range(n))
    finally:
        b.close()
    px = n * side * side
    gbs = ALG_BYTES_PER_PX * px / us / 1e3
    return {"workload": "16 textures of 2048x2048 (8 BC1, 8 ETC1s), one goofy_gpu_batch_encode call each",
            "tile": [512, 2, 1024, 1], "mean_call_us": round(us, 2), "mpix_s": round(px / us, 1),
            "hbm_gbs": round(gbs, 1), "frac": round(gbs / read_peaks()[0], 4), "outputs_equal_across_calls": same}


def run_pair(args, g, torch, src, dst, codecs, stream, device):
    """The timed step's two images (BC1 of one copy, ETC1s of the other) in
    one batch launch instead of two image launches: the bandwidth-bound BC1
    blocks and the ALU-bound ETC1s blocks share the GPU.  Outputs checked
    against the image kernels' blocks."""
    sh = stream.cuda_stream
    outs = [torch.empty_like(dst[c]) for c in codecs]
    arr = g.images_array([(src[c].data_ptr(), outs[c].data_ptr(), W, H, 4 * W, c) for c in codecs])
    b = g.Batch(2, device)
    try:
        if not args.no_autotune:
            b.autotune(arr, reps=3)
        for _ in range(3):
            assert b.encode(arr, sh) == g.OK, g.last_error()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            b.encode(arr, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        tile = list(b.get_tile())
    finally:
        b.close()
    px = 2 * W * H
    return {"api": "goofy_gpu_batch_encode: both 8192x8192 images in one launch (descriptors passed as the "
                   "kernel's parameter)",
            "ms_per_step": round(ms, 4), "mpix_s": round(px / (ms / 1e3) / 1e6, 1),
            "hbm_gbs": round(ALG_BYTES_PER_PX * px / (ms / 1e3) / 1e9, 1), "tile": tile,
            "bit_exact_vs_image_kernels": all(bool(torch.equal(outs[c], dst[c])) for c in codecs)}


def run_both(args, g, torch, img, src, dst, codecs, stream):
    """The two-codec pass (goofy_gpu_compress_both_*): BC1 and ETC1s blocks of
    the 8192x8192 scene from one read of it.  Device: K launches back to back
    between two events, inputs alternating between the two 256 MiB copies and
    outputs between two buffers; 5 algorithmic B/px (4 read, 0.5 + 0.5
    written).  Host: the same through the synchronous host call from pinned
    buffers, copies over the host link inside the region.  Both checked
    bit-exact against the single-codec outputs of the timed step."""
    import ctypes

    import numpy as np

    sh = stream.cuda_stream
    n = g.out_size(W, H)
    outs = [torch.empty(2 * n, dtype=torch.uint8, device=src[0].device) for _ in range(2)]
    tuned = None
    if not args.no_autotune:
        tile, us = g.autotune(g.CODEC_BOTH, outs[0].data_ptr(), src[0].data_ptr(), W, H, 4 * W, reps=7)
        tuned = {"tile": list(tile), "median_us": round(us, 2)}

    def launch(k):
        o = outs[k % 2].data_ptr()
        rc = g.compress_both_device(o, o + n, src[k % 2].data_ptr(), W, H, 4 * W, sh)
        if rc != g.OK:
            raise RuntimeError("compress_both_device: %s %s" % (g.status_string(rc), g.last_error()))

    for k in range(4):
        launch(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        launch(k)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    exact = all(bool(torch.equal(outs[k][:n], dst[codecs[0]]) and torch.equal(outs[k][n:], dst[codecs[1]]))
                for k in range(2))
    res = {"api": "goofy_gpu_compress_both_device: BC1 + ETC1s blocks of one image from one read of it",
           "tile": list(g.get_tile(g.CODEC_BOTH)), "autotune": tuned, "mean_launch_us": round(1e3 * ms, 2),
           "image_mpix_s": round(W * H / (ms / 1e3) / 1e6, 1),
           "codec_mpix_s": round(2 * W * H / (ms / 1e3) / 1e6, 1),
           "hbm_gbs": round(5.0 * W * H / (ms / 1e3) / 1e9, 1), "algorithmic_bytes_per_px": 5.0,
           "bit_exact_vs_single_codec": exact}
    if args.no_e2e:
        return res
    nbytes = img.size
    p_in, p_out = g.host_alloc(nbytes), g.host_alloc(2 * n)
    try:
        np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(p_in))[:] = img.reshape(-1)
        for _ in range(2):
            assert g.compress_both_host(p_out, p_out + n, p_in, W, H, 4 * W) == g.OK, g.last_error()
        steps = max(3, min(args.steps, 20))
        t0 = time.perf_counter()
        for _ in range(steps):
            rc = g.compress_both_host(p_out, p_out + n, p_in, W, H, 4 * W)
            if rc != g.OK:
                raise RuntimeError(g.last_error())
        dt = (time.perf_counter() - t0) / steps
        host = np.ctypeslib.as_array((ctypes.c_uint8 * (2 * n)).from_address(p_out))
        exact_host = bool(np.array_equal(host[:n], dst[codecs[0]].cpu().numpy()) and
                          np.array_equal(host[n:], dst[codecs[1]].cpu().numpy()))
    finally:
        g.host_free(p_in)
        g.host_free(p_out)
    res["e2e"] = {"api": "goofy_gpu_compress_both_host, pinned host in/out (direct path)", "steps": steps,
                  "ms_per_call": round(1e3 * dt, 3), "codec_mpix_s": round(2 * W * H / dt / 1e6, 1),
                  "h2d_bytes_per_call": nbytes, "d2h_bytes_per_call": 2 * n, "bit_exact": exact_host}
    return res


def run_two_streams(args, g, torch, src, dst, codecs, stream):
    """The timed step's two launches on two streams at once (the BC1 image
    on one, the ETC1s image on the other): the bandwidth-bound BC1 kernel and
    the ALU-bound ETC1s kernel may then share the GPU.  Step time = from the
    first launch to both finished."""
    other = torch.cuda.Stream()
    outs = [torch.empty_like(dst[c]) for c in codecs]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev_fork, ev_join = torch.cuda.Event(), torch.cuda.Event()

    def step():
        ev_fork.record(stream)
        other.wait_event(ev_fork)
        assert g.compress_device(codecs[1], outs[1].data_ptr(), src[1].data_ptr(), W, H, 4 * W,
                                 other.cuda_stream) == g.OK
        assert g.compress_device(codecs[0], outs[0].data_ptr(), src[0].data_ptr(), W, H, 4 * W,
                                 stream.cuda_stream) == g.OK
        ev_join.record(other)
        stream.wait_event(ev_join)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    px = 2 * W * H
    return {"api": "goofy_gpu_compress_*_device on two streams (ETC1s issued first)", "ms_per_step": round(ms, 4),
            "mpix_s": round(px / (ms / 1e3) / 1e6, 1), "hbm_gbs": round(ALG_BYTES_PER_PX * px / (ms / 1e3) / 1e9, 1),
            "bit_exact_vs_image_kernels": all(bool(torch.equal(outs[c], dst[c])) for c in codecs)}


def run_mips(g, torch, workloads, img, d_src, stream):
    """Device mip chain of the 8192x8192 image (levels 4096x4096 .. 4x4; up to
    6 levels per launch): mean time of 10 chains back to back, HBM rate for the algorithmic bytes (the
    image read once, every level written once) and equality with the host
    chain."""
    nbytes = g.lib().goofy_gpu_mip_arena_bytes(W, H)
    arena = torch.empty(nbytes + 256, dtype=torch.uint8, device=d_src.device)
    base = arena.data_ptr() + (-arena.data_ptr()) % 256
    sh = stream.cuda_stream
    for _ in range(3):
        levels = g.generate_mips(d_src, W, H, 4 * W, base, nbytes, sh)
    e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_a.record(stream)
    for _ in range(10):  # 10 chains back to back between two events
        levels = g.generate_mips(d_src, W, H, 4 * W, base, nbytes, sh)
    e_b.record(stream)
    e_b.synchronize()
    ms = e_a.elapsed_time(e_b) / 10
    moved = 4 * W * H + sum(4 * lw * lh for (_, lw, lh, _) in levels[1:])  # read the image once, write every level
    host = arena.cpu().numpy()
    off0 = base - arena.data_ptr()
    exact, cur, cw, ch = True, img, W, H
    for (ptr, lw, lh, pitch) in levels[1:]:
        cur, cw, ch = workloads.downsample(cur, cw, ch)
        o = off0 + (ptr - base)
        exact = exact and bool((host[o:o + pitch * lh].reshape(lh, pitch)[:, :4 * lw] == cur).all())
    return {"workload": "mip chain of the 8192x8192 scene, levels 4096x4096 .. 4x4 (2x2 box with rounding)",
            "levels": len(levels) - 1, "us": round(ms * 1e3, 2),
            "bytes_moved": moved, "hbm_gbs": round(moved / (ms / 1e3) / 1e9, 1), "bit_exact_vs_host_chain": exact}


def run_batched(args, g, torch, stream, dev):
    """Mixed batch: `--batch-textures` textures (64..2048 per side, 20% with
    mip chains, BC1 / ETC1s 50/50), every level resident in HBM.  Batched =
    one persistent launch per step (autotuned tile, CUDA-graph replay); plain
    = one image-kernel launch per texture level, back to back on one stream."""
    import numpy as np

    from goofy_gb300 import workloads

    t0 = time.perf_counter()
    levels = workloads.texture_batch(args.batch_textures)
    gen_s = time.perf_counter() - t0
    pixels = sum(lv["width"] * lv["height"] for lv in levels)
    in_bytes = sum((lv["pixels"].size + 255) // 256 * 256 for lv in levels)
    out_sizes = [g.out_size(lv["width"], lv["height"]) for lv in levels]
    arena_in = torch.empty(in_bytes, dtype=torch.uint8, device=dev)
    outs = [torch.zeros(sum(out_sizes), dtype=torch.uint8, device=dev) for _ in range(2)]
    descs = [[], []]
    off_in = off_out = 0
    for lv, n in zip(levels, out_sizes):
        px = lv["pixels"]
        arena_in[off_in:off_in + px.size] = torch.from_numpy(np.ascontiguousarray(px).reshape(-1)).to(dev)
        for k in range(2):
            descs[k].append((arena_in.data_ptr() + off_in, outs[k].data_ptr() + off_out, lv["width"], lv["height"],
                             px.strides[0], lv["codec"]))
        off_in += (px.size + 255) // 256 * 256
        off_out += n
    sh = stream.cuda_stream
    reps = 5
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def plain_pass(k):
        for d in descs[k]:
            rc = g.compress_device(d[5], d[1], d[0], d[2], d[3], d[4], sh)
            if rc != g.OK:
                raise RuntimeError(g.last_error())

    plain_pass(0)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        plain_pass(0)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / reps
    plain_launches = len(descs[0])

    b = g.Batch(len(levels), torch.cuda.current_device())
    try:
        arr = g.images_array(descs[1])
        if args.no_autotune:
            tile = b.get_tile()
        else:
            tile, _ = b.autotune(arr, reps=3)
        for _ in range(3):
            assert b.encode(arr, sh) == g.OK, g.last_error()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            b.encode(arr, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        batch_ms = e0.elapsed_time(e1) / reps
    finally:
        b.close()
    exact = bool(torch.equal(outs[0], outs[1]))
    return {"workload": "%d textures, 64..2048 px per side (log-uniform), 20%% with full mip chains, "
                        "BC1/ETC1s 50/50, content = synthetic scene seeded by texture index" % args.batch_textures,
            "levels": len(levels), "pixels": pixels, "generate_s": round(gen_s, 1),
            "batched_mpix_s": round(pixels / (batch_ms / 1e3) / 1e6, 1), "batched_ms": round(batch_ms, 4),
            "batched_hbm_gbs": round(ALG_BYTES_PER_PX * pixels / (batch_ms / 1e3) / 1e9, 1),
            "batched_tile": list(tile), "plain_mpix_s": round(pixels / (plain_ms / 1e3) / 1e6, 1),
            "plain_ms": round(plain_ms, 4), "plain_launches_per_step": plain_launches,
            "speedup_vs_plain": round(plain_ms / batch_ms, 2), "bit_exact_vs_plain": exact,
            "graphs": True}


def run_serving(args, g, device):
    """Serving: an open-loop Poisson stream of host-memory requests (sizes of
    the mixed batch's texture levels plus a 1024x1024 probe class at 10% of
    arrivals, BC1 / ETC1s 50/50, pinned inputs and outputs), offered at
    10/25/50/75/90% of the server's measured capacity.  Capacity = the same
    request mix all arriving at once (best of three runs, after a warm-up).  Both data paths of the server are run;
    the plain loop (one request per launch, sequential) is the baseline."""
    import numpy as np

    from goofy_gb300 import workloads

    rng = np.random.default_rng(4)
    specs = [(lv["width"], lv["height"]) for lv in workloads.texture_batch(1000, with_pixels=False)]
    sizes = sorted(set(specs) | {(1024, 1024)})
    pinned = []

    def pin(nbytes):
        arr, ptr = g.pinned_array(nbytes)
        pinned.append(ptr)
        return arr, ptr

    src = {}
    for (w, h) in sizes:
        arr, ptr = pin(w * h * 4)
        arr.reshape(h, 4 * w)[:] = workloads.scene(w, h, 7000 + w * 3 + h)
        src[(w, h)] = ptr
    ring_bytes = 1 << 29
    _, out_ptr = pin(ring_bytes)

    def stream(n, rate_per_s):
        """n requests: sizes, codecs, arrival offsets (ns), output offsets in the ring."""
        probe = rng.random(n) < 0.10
        pick = rng.integers(0, len(specs), n)
        wh = [(1024, 1024) if probe[i] else specs[pick[i]] for i in range(n)]
        codec = rng.integers(0, 2, n)
        if rate_per_s is None:
            arrival = np.zeros(n, np.int64)
        else:
            arrival = np.cumsum(rng.exponential(1e9 / rate_per_s, n)).astype(np.int64)
        reqs, off = [], 0
        for i in range(n):
            w, h = wh[i]
            nb = (w // 4) * (h // 4) * 8
            if off + nb > ring_bytes:
                off = 0
            reqs.append((src[(w, h)], out_ptr + off, w, h, 4 * w, int(codec[i])))
            off += (nb + 255) // 256 * 256
        return reqs, arrival, np.array([w * h for (w, h) in wh], np.int64), probe

    def tail_phases(lat_ns, stamps):
        """Where the slowest 1% of requests spent their time (means, ms):
        submitted late (the submitting thread behind schedule), queued before
        admission, admitted before launch, launch to completion."""
        tail = lat_ns >= np.percentile(lat_ns, 99)
        sub, adm, lau, done = (stamps[tail, k].astype(np.float64) for k in range(4))
        sched = done - lat_ns[tail]
        out = {k: round(float(v.mean()) / 1e6, 3) for k, v in
               (("submit_late", sub - sched), ("queued", adm - sub), ("admitted", lau - adm),
                ("launch_to_done", done - lau))}
        w = int(np.argmax(lat_ns))  # and the single slowest request, with its arrival time in the run
        st = stamps[w].astype(np.float64)
        ws = st[3] - lat_ns[w]
        first = float((stamps[:, 3] - lat_ns).min())
        out["slowest"] = {k: round(float(v) / 1e6, 3) for k, v in
                          (("submit_late", st[0] - ws), ("queued", st[1] - st[0]), ("admitted", st[2] - st[1]),
                           ("launch_to_done", st[3] - st[2]), ("arrived_at", ws - first))}
        return out

    def classes(px, probe, lat_ns):
        out = {}
        groups = {"probe_1024x1024": probe, "small_le_128x128": (~probe) & (px <= 128 * 128),
                  "medium_le_512x512": (~probe) & (px > 128 * 128) & (px <= 512 * 512),
                  "large_gt_512x512": (~probe) & (px > 512 * 512)}
        for k, m in groups.items():
            if m.any():
                v = lat_ns[m] / 1e6
                out[k] = {"n": int(m.sum()), "p50_ms": round(float(np.percentile(v, 50)), 3),
                          "p99_ms": round(float(np.percentile(v, 99)), 3)}
        return out

    result = {"workload": "open-loop Poisson requests: sizes of the 1000-texture batch's levels + 10% 1024x1024 "
                          "probe, BC1/ETC1s 50/50, pinned host in/out, device budget 16 GiB",
              "offered_load_basis": "fraction of the server's own measured capacity (all requests arriving at "
                                    "once); every request crosses the host link, whose measured H2D ceiling "
                                    "(~211 GB/s) caps serving far below the device-resident batched rate",
              "host_cpus": os.cpu_count(), "cgroup_cpu_quota": cpu_quota()}
    try:
        # the direct server learns of each launch's end from a thread waiting on its last event (no host
        # function between its launches on the one stream); the staged one from a host callback
        for name, mode, comp in (("staged", g.SERVER_STAGED, g.COMPLETION_CALLBACK),
                                 ("direct", g.SERVER_DIRECT, g.COMPLETION_EVENT)):
            srv = g.Server(mode=mode, device=device, completion=comp)
            try:
                n_sat = 20000
                reqs, arrival, px, probe = stream(n_sat, None)
                assert srv.replay(reqs[:2000], arrival[:2000])[0] == g.OK  # the server's first launches
                caps = []
                for _ in range(3):
                    rc, lat, wall = srv.replay(reqs, arrival)
                    assert rc == g.OK, g.last_error()
                    caps.append(float(px.sum()) / (wall / 1e9))
                cap = max(caps)
                entry = {"completion": "event" if comp == g.COMPLETION_EVENT else "callback",
                         "capacity_mpix_s": round(cap / 1e6, 1), "capacity_requests": n_sat,
                         "capacity_runs_mpix_s": [round(c / 1e6, 1) for c in caps],
                         "mean_request_px": round(float(px.mean()))}
                warm_rate = 0.1 * cap / float(px.mean())  # settle the server before the measured runs
                reqs, arrival, _, _ = stream(max(200, int(warm_rate * 0.2)), warm_rate)
                assert srv.replay(reqs, arrival)[0] == g.OK
                loads = {}
                for f in (0.10, 0.25, 0.50, 0.75, 0.90):
                    rate = f * cap / float(px.mean())
                    n = max(200, int(rate * args.serve_seconds))
                    reqs, arrival, rpx, rprobe = stream(n, rate)
                    thr0, psi0 = cpu_throttle_stats(), pressure_totals()
                    srv.stats()  # resets the slowest-launch figures
                    rc, lat, wall, stamps = srv.replay(reqs, arrival, with_times=True)
                    thr1, psi1, st = cpu_throttle_stats(), pressure_totals(), srv.stats()
                    assert rc == g.OK, g.last_error()
                    loads["%d%%" % round(100 * f)] = {
                        "offered_mpix_s": round(f * cap / 1e6, 1), "requests": n,
                        "sustained_mpix_s": round(float(rpx.sum()) / (wall / 1e9) / 1e6, 1),
                        "p50_ms": round(float(np.percentile(lat, 50)) / 1e6, 3),
                        "p99_ms": round(float(np.percentile(lat, 99)) / 1e6, 3),
                        "p999_ms": round(float(np.percentile(lat, 99.9)) / 1e6, 3),
                        "max_ms": round(float(lat.max()) / 1e6, 3),
                        "by_class": classes(rpx, rprobe, lat), "p99_tail_phases_ms": tail_phases(lat, stamps),
                        **window_diagnostics(thr0, psi0, thr1, psi1, st)}
                entry["loads"] = loads
                if mode == g.SERVER_STAGED and args.serve_soak_s > 0:
                    # one long low-load window: the rare stalls show in its max
                    rate = 0.10 * cap / float(px.mean())
                    reqs, arrival, rpx, _ = stream(max(200, int(rate * args.serve_soak_s)), rate)
                    thr0, psi0 = cpu_throttle_stats(), pressure_totals()
                    srv.stats()
                    rc, lat, wall = srv.replay(reqs, arrival)
                    thr1, psi1, st = cpu_throttle_stats(), pressure_totals(), srv.stats()
                    assert rc == g.OK, g.last_error()
                    entry["soak_10pct"] = {
                        "seconds": args.serve_soak_s, "requests": len(reqs),
                        "p50_ms": round(float(np.percentile(lat, 50)) / 1e6, 3),
                        "p99_ms": round(float(np.percentile(lat, 99)) / 1e6, 3),
                        "p999_ms": round(float(np.percentile(lat, 99.9)) / 1e6, 3),
                        "max_ms": round(float(lat.max()) / 1e6, 3), "over_3ms": int((lat > 3e6).sum()),
                        **window_diagnostics(thr0, psi0, thr1, psi1, st)}
                entry["stats"] = srv.stats()
                result[name] = entry
            finally:
                srv.close()
        # the staged server with per-request quality (RGB PSNR of every request, measured on the GPU)
        srv = g.Server(mode=g.SERVER_STAGED, device=device, quality=True)
        try:
            reqs, arrival, px, _ = stream(20000, None)
            srv.replay(reqs[:2000], arrival[:2000])
            rc, lat, wall, _ = srv.replay(reqs, arrival, with_times=True)
            assert rc == g.OK, g.last_error()
            ps = srv.last_psnr
            result["staged_with_quality"] = {
                "capacity_mpix_s": round(float(px.sum()) / (wall / 1e9) / 1e6, 1), "requests": len(reqs),
                "psnr_rgb_db_mean": round(float(ps.mean()), 4), "psnr_rgb_db_min": round(float(ps.min()), 4),
                "note": "one more launch per batch decodes the fresh blocks and sums the harness's errors"}
        finally:
            srv.close()
        n_plain = 4000
        reqs, arrival, px, probe = stream(n_plain, None)
        assert g.plain_replay(reqs[:400], arrival[:400], device)[0] == g.OK
        rc, lat, wall = g.plain_replay(reqs, arrival, device)
        assert rc == g.OK, g.last_error()
        plain_cap = float(px.sum()) / (wall / 1e9)
        best = max(result["staged"]["capacity_mpix_s"], result["direct"]["capacity_mpix_s"])
        result["plain"] = {"capacity_mpix_s": round(plain_cap / 1e6, 1), "requests": n_plain,
                           "server_vs_plain": round(best * 1e6 / plain_cap, 2)}
        f = 0.5
        rate = f * plain_cap / float(px.mean())
        n = max(200, int(rate * args.serve_seconds))
        reqs, arrival, rpx, rprobe = stream(n, rate)
        rc, lat, wall = g.plain_replay(reqs, arrival, device)
        result["plain"]["at_50pct_of_own_capacity"] = {
            "p50_ms": round(float(np.percentile(lat, 50)) / 1e6, 3),
            "p99_ms": round(float(np.percentile(lat, 99)) / 1e6, 3), "by_class": classes(rpx, rprobe, lat)}
    finally:
        for p in pinned:
            g.host_free(p)
    return result


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    # nothing of the GPU library is built or loaded on this arm: the scene comes
    # from the generator compiled into the oracle library
    import oracle
    from oracle import build as oracle_build

    oracle_build.build()
    img = oracle.scene(W, H, SEED, PERIOD_SCALE, RECTS, threads=0)
    fn, kind, label = oracle.ref_encoder()
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_encode_all(fn, img, cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_encode_all(fn, img, cores)
    dt = time.perf_counter() - t0
    value = 2 * W * H * args.steps / dt / 1e6
    line = {"metric": METRIC, "value": round(value, 1), "unit": "MPix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic", "impl": "reference",
            "config": dict(CONFIG), "implementation": label,
            "cpu_baseline": {"value": round(value, 1), "unit": "MPix/s", "cores": cores, "kind": kind,
                             "implementation": label, "cpu": "%s, %s" % (cpu_model(), platform.machine()),
                             "sample": "full 8192x8192 image per step, BC1 + ETC1s, block rows striped over "
                                       "%d threads" % cores},
            "e2e": {"value": round(value, 1), "unit": "MPix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    import goofy_gb300 as g
    from goofy_gb300 import build as lib_build
    from goofy_gb300 import workloads

    lib_build.build()
    assert g.init(local) == g.OK, g.last_error()
    img = workloads.scene(W, H, SEED, PERIOD_SCALE, RECTS, threads=0)
    nbytes = img.size
    dev = torch.device("cuda", local)
    src = [torch.from_numpy(img.reshape(-1)).to(dev), None]
    src[1] = src[0].clone()
    n_out = g.out_size(W, H)
    dst = [torch.empty(n_out, dtype=torch.uint8, device=dev) for _ in range(2)]
    scratch = [torch.empty(n_out, dtype=torch.uint8, device=dev) for _ in range(2)]
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    codecs = (g.CODEC_BC1, g.CODEC_ETC1S)

    def step():
        for c in codecs:
            rc = g.compress_device(c, dst[c].data_ptr(), src[c].data_ptr(), W, H, 4 * W, sh)
            if rc != g.OK:
                raise RuntimeError("encode failed: %s %s" % (g.status_string(rc), g.last_error()))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    names = {g.CODEC_BC1: "bc1", g.CODEC_ETC1S: "etc1s"}
    tuned = {}
    if args.sweep:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for c in codecs:
            for threads, bpt, pers in [(t, b, p) for p in (0, 1, 2) for t in (128, 256, 512) for b in (1, 2, 4)
                                       if not (p and b == 4)]:
                    g.set_tile(c, threads, bpt, pers)
                    ts = []
                    for r in range(9):
                        e0.record(stream)
                        g.compress_device(c, dst[c].data_ptr(), src[c].data_ptr(), W, H, 4 * W, sh)
                        e1.record(stream)
                        e1.synchronize()
                        ts.append(e0.elapsed_time(e1) * 1e3)
                    print("sweep %s threads=%d bpt=%d persistent=%d median_us=%.2f min_us=%.2f" % (
                        names[c], threads, bpt, pers, statistics.median(ts), min(ts)), file=sys.stderr)
    # tuned tiles go to a cache file of this run (the library's per-user default is left alone)
    import tempfile

    cache_dir = tempfile.mkdtemp(prefix="goofy_tiles_")
    g.set_tile_cache_path(os.path.join(cache_dir, "tiles.txt"))
    if not args.no_autotune:
        # the step alternates the codecs, so the pair is tuned together (goofy_gpu_autotune_pair)
        t_bc1, t_etc1s, us = g.autotune_pair(dst[0].data_ptr(), dst[1].data_ptr(), src[0].data_ptr(), W, H, 4 * W,
                                             reps=7)
        tuned = {"bc1": list(t_bc1), "etc1s": list(t_etc1s), "pair_us": round(us, 2),
                 "api": "goofy_gpu_autotune_pair (alternating BC1 / ETC1s launches)"}

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    with ClockSampler(local) as clocks:
        t_soak = time.perf_counter()
        while time.perf_counter() - t_soak < args.soak_s:
            for _ in range(20):
                step()
            torch.cuda.synchronize()
        # timed region: K steps, CUDA events on the launching stream at its two ends only (an event
        # recorded between two launches delays the second one's start by a few microseconds)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        start.record(stream)
        for k in range(args.steps):
            step()
        end.record(stream)
        torch.cuda.synchronize()
        barrier()
        # each kernel's launch duration: K launches of it back to back between two events, the
        # inputs alternating between the two 256 MiB copies (larger than L2 either way) and the
        # outputs between two scratch buffers (no launch rewrites the lines the previous one wrote)
        per_launch = {}
        for c in codecs:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for k in range(args.steps):
                g.compress_device(c, scratch[k % 2].data_ptr(), src[(c + k) % 2].data_ptr(), W, H, 4 * W, sh)
            e1.record(stream)
            torch.cuda.synchronize()
            per_launch[c] = e0.elapsed_time(e1) / args.steps
    total_ms = start.elapsed_time(end)
    total_ms = max_over_ranks(total_ms, world)

    # the tile cache as a new process's first call sees it: defaults back, the
    # tuned tiles read from the file again, the same K steps timed with them
    tile_cache = None
    if not args.no_autotune:
        tuned_tiles = {names[c]: list(g.get_tile(c)) for c in codecs}
        g.reset_tiles()
        reloaded = g.load_tile_cache(local)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(3):
            step()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        cached_ms = e0.elapsed_time(e1) / args.steps
        tile_cache = {"tiles_tuned": tuned_tiles, "tiles_after_reload": {names[c]: list(g.get_tile(c)) for c in codecs},
                      "entries_installed": reloaded, "step_us_tuned": round(1e3 * total_ms / args.steps, 2),
                      "step_us_cached": round(1e3 * cached_ms, 2),
                      "cached_over_tuned": round(cached_ms / (total_ms / args.steps), 4),
                      "note": "after goofy_gpu_reset_tiles + goofy_gpu_load_tile_cache, as the first call of a new "
                              "process installs them (cache file of this run)"}

    px_per_step = 2 * W * H
    value = job_rate_mpix_s(world, px_per_step, args.steps, total_ms)

    # e2e through the host C ABI from pinned memory
    e2e = None
    if not args.no_e2e:
        import ctypes

        p_in = g.host_alloc(nbytes)
        p_out = g.host_alloc(n_out)
        try:
            np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(p_in))[:] = img.reshape(-1)
            for _ in range(2):
                for c in codecs:
                    assert g.compress_host(c, p_out, p_in, W, H, 4 * W) == g.OK, g.last_error()
            e2e_steps = max(3, min(args.steps, 20))

            def e2e_rate(out_ptr, in_ptr, steps):
                barrier()
                t0 = time.perf_counter()
                for _ in range(steps):
                    for c in codecs:
                        rc = g.compress_host(c, out_ptr, in_ptr, W, H, 4 * W)
                        if rc != g.OK:
                            raise RuntimeError(g.last_error())
                dt = max_over_ranks(time.perf_counter() - t0, world)
                return job_rate_mpix_s(world, px_per_step, steps, 1e3 * dt)

            value_e2e = e2e_rate(p_out, p_in, e2e_steps)
            g.set_host_path(g.HOST_PATH_STAGED)
            e2e_rate(p_out, p_in, 1)
            staged_e2e = e2e_rate(p_out, p_in, e2e_steps)
            g.set_host_path(g.HOST_PATH_AUTO)
            page_in = np.ascontiguousarray(img.reshape(-1))
            page_out = np.empty(n_out, np.uint8)
            e2e_rate(page_out.ctypes.data, page_in.ctypes.data, 1)
            pageable_e2e = e2e_rate(page_out.ctypes.data, page_in.ctypes.data, e2e_steps)
            dropin = run_dropin_latency(g, img) if world == 1 else None
            e2e = {"value": round(value_e2e, 1), "unit": "MPix/s",
                   "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": 2 * n_out, "steps": e2e_steps,
                   "api": "goofy_gpu_compress_host (the engine of goofy::compressDXT1/ETC1), pinned host in/out, "
                          "default path selection (direct: the kernel reads / writes the host buffers over "
                          "NVLink-C2C)",
                   "staged_path_mpix_s": round(staged_e2e, 1), "pageable_buffers_mpix_s": round(pageable_e2e, 1),
                   "host_link_bound_mpix_s": "about 52700 (measured H2D ceiling ~211 GB/s at 4 B/px)",
                   "dropin_call_us": dropin}
        finally:
            g.host_free(p_in)
            g.host_free(p_out)

    if rank != 0:
        import shutil

        shutil.rmtree(cache_dir, ignore_errors=True)
        torch.distributed.destroy_process_group()
        return 0

    peak, peak_kind = read_peaks()
    per_codec = {}
    for c in codecs:
        ms = per_launch[c]
        per_codec[names[c]] = {"mean_launch_us": round(1e3 * ms, 2),
                               "mpix_s": round(W * H / (ms / 1e3) / 1e6, 1),
                               "hbm_gbs": round(ALG_BYTES_PER_PX * W * H / (ms / 1e3) / 1e9, 1)}
    per_codec["timing"] = ("mean of %d launches of the kernel back to back between two CUDA events, right after "
                           "the timed steps, inputs and outputs alternating between two buffers each; the step "
                           "(%.2f us) also holds the switch from one kernel to the other" % (args.steps,
                                                                                           1e3 * total_ms / args.steps))
    dom = max(codecs, key=lambda c: per_launch[c])
    dom_ms = per_launch[dom]
    achieved = ALG_BYTES_PER_PX * W * H / (dom_ms / 1e3) / 1e9
    kernel = "encode_image_tma" if g.get_tile(dom)[2] == 2 else "encode_image_kernel"
    traffic = read_traffic("%s_%s_8192" % (kernel, names[dom]))
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": "%s<%s>" % (kernel, names[dom]),
                "algorithmic_bytes_per_launch": int(ALG_BYTES_PER_PX * W * H),
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s"}
    cpu = None
    # quality: RGB PSNR of the timed outputs (the reference harness's secondary
    # metric), and the speed of the fused decode + squared-error kernel
    quality = {}
    d_sums = torch.zeros(6, dtype=torch.int64, device=dev)
    for c in codecs:
        rc, psnr, sums = g.psnr_rgb(c, dst[c], src[c], W, H, 4 * W)
        assert rc == g.OK, g.last_error()
        # 10 launches back to back between two events (the sums only accumulate), after 2 untimed
        for r in range(2):
            g.block_error_device(c, dst[c], src[(c + 1) % 2], W, H, 4 * W, d_sums, sh)
        e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_a.record(stream)
        for r in range(10):
            g.block_error_device(c, dst[c], src[(c + r) % 2], W, H, 4 * W, d_sums, sh)
        e_b.record(stream)
        e_b.synchronize()
        ms = e_a.elapsed_time(e_b) / 10
        quality[names[c]] = {"psnr_rgb_db": round(psnr, 5), "unsupported_blocks": int(sums[4]),
                             "decode_error_kernel_us": round(ms * 1e3, 2),
                             "decode_error_hbm_gbs": round(ALG_BYTES_PER_PX * W * H / (ms / 1e3) / 1e9, 1)}
    # the per-GPU feature sections run at N = 1 only: with several ranks they
    # would repeat on every GPU and contend for the shared host cores
    single = world == 1
    mips = run_mips(g, torch, workloads, img, src[0], stream) if single else None
    pair = run_pair(args, g, torch, src, dst, codecs, stream, local) if single else None
    batch16 = run_batch_16x2048(args, g, torch, workloads, stream, local) if single else None
    two_streams = run_two_streams(args, g, torch, src, dst, codecs, stream) if single else None
    both = run_both(args, g, torch, img, src, dst, codecs, stream) if single else None
    small = run_small_configs(args, g, torch, workloads, codecs, stream, peak) if single else None
    batched = None
    if not args.no_batched and single:
        batched = run_batched(args, g, torch, stream, dev)
    serving = None
    if not args.no_serving and single:
        serving = run_serving(args, g, local)
    if not args.no_cpu and rank == 0 and world == 1:
        from oracle import build as oracle_build

        oracle_build.build()
        cpu = cpu_baseline(img, [dst[c].cpu().numpy() for c in codecs])
    tiles = {names[c]: list(g.get_tile(c)) for c in codecs}
    line = {"metric": METRIC, "value": round(value, 1), "unit": "MPix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": dict(CONFIG), "per_gpu": "same workload on every GPU", "tiles": tiles, "autotune": tuned or None,
            "serving": serving, "per_codec": per_codec, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "quality": quality, "mips": mips, "pair_batched": pair, "two_streams": two_streams,
            "both_codecs_one_pass": both, "small_configs": small, "batch_16x2048": batch16, "batched": batched, "tile_cache": tile_cache,
            "clocks": dict(clocks.summary(), window="timed region + %.1f s soak of the same loop" % args.soak_s),
            "gpu_launches": 2 * args.steps}
    line["summary"] = summary(line, peak)
    import shutil

    g.set_tile_cache_path(None)
    shutil.rmtree(cache_dir, ignore_errors=True)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_profile(args):
    """A few launches of one kernel family on a --profile-size scene,
    default tiles, nothing timed: the workload of the ncu captures under
    profiles/ (small enough for a full capture to end in a minute)."""
    import numpy as np
    import torch

    import goofy_gb300 as g
    from goofy_gb300 import build as lib_build
    from goofy_gb300 import workloads

    lib_build.build()
    assert g.init(0) == g.OK, g.last_error()
    if args.profile == "batch-pipeline":  # 16 textures of 2048x2048 (8 per codec), the pipelined tile, three launches
        side, n = 2048, 16
        img = workloads.scene(side, side, 3, threads=0)
        keep, descs = [], []
        for i in range(n):
            src = torch.from_numpy(img.reshape(-1)).cuda()
            out = torch.empty(g.out_size(side, side), dtype=torch.uint8, device="cuda")
            keep += [src, out]
            descs.append((src.data_ptr(), out.data_ptr(), side, side, 4 * side, i % 2))
        b = g.Batch(n)
        try:
            assert b.set_tile(512, 2, 1024, 1) == g.OK
            arr = g.images_array(descs)
            for _ in range(3):
                assert b.encode(arr, torch.cuda.current_stream().cuda_stream) == g.OK, g.last_error()
            torch.cuda.synchronize()
        finally:
            b.close()
        print(json.dumps({"profile": "batch-pipeline", "textures": n, "side": side,
                          "pipeline_timeouts": g.pipeline_timeouts()}))
        return 0
    if args.profile == "batch":  # the mixed batch of --batch-textures textures, three launches, default tile
        levels = workloads.texture_batch(args.batch_textures)
        keep, descs = [], []
        for lv in levels:
            src = torch.from_numpy(np.ascontiguousarray(lv["pixels"]).reshape(-1)).cuda()
            out = torch.empty(g.out_size(lv["width"], lv["height"]), dtype=torch.uint8, device="cuda")
            keep += [src, out]
            descs.append((src.data_ptr(), out.data_ptr(), lv["width"], lv["height"], lv["pixels"].strides[0],
                          lv["codec"]))
        b = g.Batch(len(descs))
        try:
            arr = g.images_array(descs)
            for _ in range(3):
                assert b.encode(arr, torch.cuda.current_stream().cuda_stream) == g.OK, g.last_error()
            torch.cuda.synchronize()
        finally:
            b.close()
        print(json.dumps({"profile": "batch", "textures": args.batch_textures, "levels": len(descs)}))
        return 0
    w, _, h = args.profile_size.partition("x")
    w = int(w)
    h = int(h) if h else w
    img = workloads.scene(w, h, SEED, w // 256, max(8, w * h // 32768), threads=0)
    src = torch.from_numpy(img.reshape(-1)).cuda()
    sh = torch.cuda.current_stream().cuda_stream
    dst = [torch.empty(g.out_size(w, h), dtype=torch.uint8, device="cuda") for _ in range(2)]
    for c in (g.CODEC_BC1, g.CODEC_ETC1S):
        for _ in range(3 if args.profile == "encode" else 1):
            assert g.compress_device(c, dst[c].data_ptr(), src.data_ptr(), w, h, 4 * w, sh) == g.OK, g.last_error()
    if args.profile == "both":
        for _ in range(3):
            assert g.compress_both_device(dst[0], dst[1], src, w, h, 4 * w, sh) == g.OK, g.last_error()
    if args.profile == "quality":
        sums = torch.zeros(6, dtype=torch.int64, device="cuda")
        rgba = torch.empty(w * h * 4, dtype=torch.uint8, device="cuda")
        bad = torch.zeros(1, dtype=torch.int64, device="cuda")
        for c in (g.CODEC_BC1, g.CODEC_ETC1S):
            for _ in range(3):
                assert g.block_error_device(c, dst[c], src, w, h, 4 * w, sums, sh) == g.OK, g.last_error()
            assert g.decode_device(c, rgba, 4 * w, dst[c], w, h, bad, sh) == g.OK, g.last_error()
    if args.profile == "mips":
        nbytes = g.lib().goofy_gpu_mip_arena_bytes(w, h)
        arena = torch.empty(nbytes + 256, dtype=torch.uint8, device="cuda")
        base = arena.data_ptr() + (-arena.data_ptr()) % 256
        for _ in range(3):
            g.generate_mips(src, w, h, 4 * w, base, nbytes, sh)
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "size": [w, h], "pipeline_timeouts": g.pipeline_timeouts()}))
    return 0


def main():
    args = parse()
    if args.profile:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
