"""Recipe: compile the reference's benchmark harness (Src/main.cpp with
Src/decoder.cpp and Src/goofy_tc_reference.cpp; the third-party encoders and
lodepng it includes come in through main.cpp) straight from the reference
tree with g++, run it once on its default test list (parrot_red) and return
its result rows.  TEST INFRASTRUCTURE ONLY: used to pin the oracle's and the
library's quality numbers (getMsePsnr) to the harness's own output.

Everything it writes stays under oracle/_ref/harness/: the binary, a
`test-data` link to the reference's photographs and the `test-results/`
folder the harness fills (result table, DDS / KTX files, TGA images).
x86-64 only (the harness and goofy_tc.h use SSE intrinsics).
"""
import os
import platform
import subprocess

from .build import REFERENCE

HERE = os.path.dirname(os.path.abspath(__file__))
RUN_DIR = os.path.join(HERE, "_ref", "harness")
BINARY = os.path.join(RUN_DIR, "goofy_harness")
FIELDS = ("image", "encoder", "format", "pixels", "time_us", "mps", "mse_r", "mse_g", "mse_b", "mse_max", "mse_rgb",
          "mse_y", "psnr_r", "psnr_g", "psnr_b", "psnr_min", "psnr_rgb", "psnr_y", "delta_min", "delta_rgb",
          "delta_y")


def available():
    return os.path.exists(os.path.join(REFERENCE, "Src", "main.cpp")) and platform.machine() in ("x86_64", "AMD64")


def build():
    os.makedirs(RUN_DIR, exist_ok=True)
    src = [os.path.join(REFERENCE, "Src", f) for f in ("main.cpp", "decoder.cpp", "goofy_tc_reference.cpp")]
    if not os.path.exists(BINARY) or any(os.path.getmtime(s) > os.path.getmtime(BINARY) for s in src):
        subprocess.run(["g++", "-O2", "-DNDEBUG", "-std=c++17", "-msse4.1", "-o", BINARY] + src + ["-lpthread"],
                       check=True)
    return BINARY


def run(timeout=900):
    """Result rows of one harness run: a list of dicts keyed by FIELDS."""
    build()
    link = os.path.join(RUN_DIR, "test-data")
    if not os.path.islink(link):
        os.symlink(os.path.join(REFERENCE, "test-data"), link)
    os.makedirs(os.path.join(RUN_DIR, "test-results"), exist_ok=True)
    subprocess.run([BINARY], cwd=RUN_DIR, check=True, timeout=timeout, stdout=subprocess.DEVNULL)
    rows = []
    with open(os.path.join(RUN_DIR, "test-results", "results.txt")) as f:
        next(f)
        for line in f:
            parts = line.strip().split(";")
            if len(parts) == len(FIELDS):
                rows.append(dict(zip(FIELDS, parts)))
    return rows


if __name__ == "__main__":
    for r in run():
        print(";".join(r[k] for k in FIELDS))
