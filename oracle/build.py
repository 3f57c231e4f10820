"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libgoofy_oracle.so`` -- the C restatement in goofy_oracle.c.
  Built on every machine (plain gcc, no SIMD intrinsics, so x86-64 and aarch64
  give the same bits).
* ``oracle/_ref/libgoofy_ref.so`` -- the reference encoder itself, compiled from
  GoofyTC/goofy_tc.h where it lies in the reference tree, through ref_shim.cpp.
  Only where that tree exists and the host is x86-64 (the header includes
  <emmintrin.h> unconditionally, goofy_tc.h:16 and :29).  Never copied.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_HEADER_DIR = "/root/reference/GoofyTC"
REFERENCE_SRC_DIR = "/root/reference/Src"
REFERENCE_PNG_DIR = "/root/reference/ThirdParty/lodepng"

ORACLE_SO = os.path.join(BUILD_DIR, "libgoofy_oracle.so")
REF_SO = os.path.join(REF_DIR, "libgoofy_ref.so")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def oracle_cmd():
    src = os.path.join(HERE, "goofy_oracle.c")
    return [src, os.path.join(HERE, "goofy_oracle.h")], [
        "gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
        "-Wall", "-o", ORACLE_SO, src, "-lm"]


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
