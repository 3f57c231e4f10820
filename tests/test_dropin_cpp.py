"""The C++ drop-in as a reference caller uses it: tests/dropin/harness_call.cpp
calls goofy::compressETC1 / compressDXT1 through the harness's function-pointer
type (Src/main.cpp:644), compiled against include/goofy_tc_gpu.h and linked
with the library instead of compiling goofy_tc.h.  On the CPU: it compiles,
links and gets the reference's return codes for bad sizes.  On the GPU: its
output files equal the golden vectors."""
import os
import subprocess

import numpy as np
import pytest

import goofy_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("dropin") / "harness_call")
    libdir = os.path.dirname(g.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "harness_call.cpp"), "-o", exe, "-L", libdir,
           "-l:" + os.path.basename(g.LIB_PATH), "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_compiles_links_and_returns_the_reference_codes(harness):
    r = subprocess.run([harness, "codes"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    # per entry point: width % 16 -> -1, height % 4 -> -2, width 8 -> -1 (goofy_tc.h:1500-1508, :1531-1539)
    assert r.stdout.split("\n")[:2] == ["-1 -2 -1", "-1 -2 -1"]


@pytest.mark.gpu
def test_harness_call_encodes_the_golden_vectors(cuda, harness, golden, tmp_path):
    w, h = int(golden["kat_width"]), int(golden["kat_height"])
    img = np.ascontiguousarray(golden["kat_input"])
    src = tmp_path / "in.rgba"
    src.write_bytes(img.tobytes())
    out_etc, out_dxt = tmp_path / "out.etc", tmp_path / "out.dxt"
    r = subprocess.run([harness, "encode", str(src), str(w), str(h), str(img.strides[0]), str(out_etc),
                        str(out_dxt)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
    assert out_etc.read_bytes() == golden["kat_etc1s"].tobytes()
    assert out_dxt.read_bytes() == golden["kat_bc1"].tobytes()
