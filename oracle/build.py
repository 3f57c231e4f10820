"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libgoofy_oracle.so`` -- the C restatement in goofy_oracle.c,
  plus the synthetic-image generator (goofy_gb300/csrc/synth.c compiled in a
  second time, so the CPU arm of the benchmark makes its input without loading
  the GPU library's files).  Built on every machine (plain gcc, no SIMD
  intrinsics, so x86-64 and aarch64 give the same bits).
* ``oracle/_ref/scalar/goofy_tc.h`` -- written here from the reference's
  GoofyTC/goofy_tc.h with its line 16 (``#define GOOFY_SSE2 (1)``) left out,
  which selects the header's own portable scalar path (goofy_tc.h:28-32,
  :398-1027) instead of SSE2.  A generated build input, never committed.
* ``oracle/_ref/libgoofy_ref_scalar.so`` -- the reference encoder compiled from
  that generated header (ref_shim.cpp, encoder part only).  It builds on any
  host where the generated header is present, including an aarch64 host
  without the reference tree, so the CPU baseline there is the reference's
  own code.
* ``oracle/_ref/libgoofy_ref.so`` -- the reference encoder itself, compiled from
  GoofyTC/goofy_tc.h where it lies in the reference tree, through ref_shim.cpp.
  Only where that tree exists and the host is x86-64: goofy_tc.h:16 defines
  GOOFY_SSE2, which selects <emmintrin.h> (:28-29) and the SSE2 path.

The reference tree is looked for at $GOOFY_REFERENCE (default below); the
test photographs at $GOOFY_TEST_DATA, else its test-data folder.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE = os.environ.get("GOOFY_REFERENCE", "/root/reference")
REFERENCE_HEADER_DIR = os.path.join(REFERENCE, "GoofyTC")
REFERENCE_SRC_DIR = os.path.join(REFERENCE, "Src")
REFERENCE_PNG_DIR = os.path.join(REFERENCE, "ThirdParty", "lodepng")
TEST_DATA = os.environ.get("GOOFY_TEST_DATA", os.path.join(REFERENCE, "test-data"))

ORACLE_SO = os.path.join(BUILD_DIR, "libgoofy_oracle.so")
REF_SO = os.path.join(REF_DIR, "libgoofy_ref.so")
SCALAR_DIR = os.path.join(REF_DIR, "scalar")
SCALAR_HEADER = os.path.join(SCALAR_DIR, "goofy_tc.h")
REF_SCALAR_SO = os.path.join(REF_DIR, "libgoofy_ref_scalar.so")
SSE2_SWITCH = "#define GOOFY_SSE2 (1)"
SSE2_SWITCH_LINE = 16
SYNTH_SRC = os.path.join(os.path.dirname(HERE), "goofy_gb300", "csrc", "synth.c")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def oracle_cmd():
    src = os.path.join(HERE, "goofy_oracle.c")
    return [src, os.path.join(HERE, "goofy_oracle.h"), SYNTH_SRC], [
        "gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
        "-Wall", "-o", ORACLE_SO, src, SYNTH_SRC, "-lm"]


def ref_available():
    return (os.path.exists(os.path.join(REFERENCE_HEADER_DIR, "goofy_tc.h"))
            and platform.machine() in ("x86_64", "AMD64"))


def ref_cmd():
    """The reference encoder header, the reference harness's decoder
    (Src/decoder.cpp) and its PNG loader (ThirdParty/lodepng/lodepng.cpp), all
    compiled from where they lie, behind ref_shim.cpp."""
    src = os.path.join(HERE, "ref_shim.cpp")
    hdr = os.path.join(REFERENCE_HEADER_DIR, "goofy_tc.h")
    dec = os.path.join(REFERENCE_SRC_DIR, "decoder.cpp")
    png = os.path.join(REFERENCE_PNG_DIR, "lodepng.cpp")
    return [src, hdr, dec, png], [
        "g++", "-O3", "-DNDEBUG", "-std=c++17", "-fPIC", "-shared", "-pthread", "-msse2",
        "-I", REFERENCE_HEADER_DIR, "-I", REFERENCE_SRC_DIR, "-I", REFERENCE_PNG_DIR, "-o", REF_SO, src, dec, png]


def write_scalar_header():
    """oracle/_ref/scalar/goofy_tc.h: the reference header without the line
    that turns SSE2 on (checked to be exactly that line), where the reference
    tree exists.  Returns whether the generated header is present."""
    src = os.path.join(REFERENCE_HEADER_DIR, "goofy_tc.h")
    if os.path.exists(src) and _stale(SCALAR_HEADER, [src]):
        lines = open(src).read().split("\n")
        if lines[SSE2_SWITCH_LINE - 1].strip() != SSE2_SWITCH:
            raise RuntimeError("goofy_tc.h:%d is not %r" % (SSE2_SWITCH_LINE, SSE2_SWITCH))
        os.makedirs(SCALAR_DIR, exist_ok=True)
        with open(SCALAR_HEADER, "w") as f:
            f.write("\n".join(lines[:SSE2_SWITCH_LINE - 1] + lines[SSE2_SWITCH_LINE:]))
    return os.path.exists(SCALAR_HEADER)


def ref_scalar_cmd():
    """The reference encoder's scalar path from the generated header."""
    src = os.path.join(HERE, "ref_shim.cpp")
    return [src, SCALAR_HEADER], [
        "g++", "-O3", "-DNDEBUG", "-DGOOFY_REF_ENCODER_ONLY", "-std=c++17", "-fPIC", "-shared", "-pthread",
        "-I", SCALAR_DIR, "-o", REF_SCALAR_SO, src]


def build(verbose=False):
    """Compile what is stale; returns the list of Popen handles' commands run."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    jobs = []
    deps, cmd = oracle_cmd()
    if _stale(ORACLE_SO, deps):
        jobs.append(cmd)
    if ref_available():
        os.makedirs(REF_DIR, exist_ok=True)
        deps, cmd = ref_cmd()
        if _stale(REF_SO, deps):
            jobs.append(cmd)
    if write_scalar_header():
        deps, cmd = ref_scalar_cmd()
        if _stale(REF_SCALAR_SO, deps):
            jobs.append(cmd)
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in jobs]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(c), out.decode(errors="replace")))
        if verbose:
            print(" ".join(c))
    return [c for c, _ in procs]


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
