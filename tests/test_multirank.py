"""The N > 1 host logic of bench.py on CPU: two gloo ranks over 127.0.0.1.
Replicas need no data-path collective; the only cross-rank steps are the
barrier and the max-over-ranks of the timings, and only rank 0 prints.  The
reference arm runs on rank 0 alone; other ranks exit without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank, world, _ = bench.dist_env()
dist.init_process_group("gloo")
slow = bench.max_over_ranks(10.0 + 5.0 * rank, world)
dist.barrier()
print(json.dumps({{"rank": rank, "world": world, "slowest_ms": slow,
                  "rate": bench.job_rate_mpix_s(world, 1000000, 4, slow)}}), flush=True)
dist.destroy_process_group()
"""

REFERENCE_ARM = r"""
import sys
sys.path.insert(0, {root!r})
import bench
bench.W, bench.H = 256, 128  # a small image keeps the CPU arm short here
sys.argv = ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1"]
sys.exit(bench.main())
"""


def _launch(code, world=2):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", code.format(root=ROOT)], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_max_over_ranks_and_job_rate():
    outs = _launch(WORKER)
    lines = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    for ln in lines:
        assert ln["world"] == 2
        assert ln["slowest_ms"] == 15.0  # rank 1's time
        assert ln["rate"] == pytest.approx(2 * 1e6 * 4 / 0.015 / 1e6)


def test_reference_arm_runs_on_rank0_only(built):
    outs = _launch(REFERENCE_ARM)
    line = json.loads(outs[0].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["value"] == line["value"]
    assert outs[1].strip() == ""
