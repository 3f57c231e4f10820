"""Build recipe of the GB300 encoder library (no cmake; nvcc + gcc only).

Outputs, all in ``goofy_gb300/_build/`` (git-ignored, rebuilt on each host):

* ``libgoofy_gb300.so`` -- CUDA kernels for sm_103a + the C ABI + the C++
  drop-in ``goofy::compressDXT1/compressETC1`` (host code in C++).
* ``libgoofy_synth.so`` -- deterministic synthetic workloads (C).

Translation units compile in parallel; a full build takes well under a minute.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libgoofy_gb300.so")
SYNTH_LIB = os.path.join(BUILD_DIR, "libgoofy_synth.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(_nvcc()))


CU_SOURCES = ["encode_kernels.cu", "encode_tma.cu", "batch_kernels.cu", "batch_noalloc.cu", "decode_kernels.cu", "mips.cu"]
CPP_SOURCES = ["capi.cpp", "tile_cache.cpp", "batch.cpp", "server.cpp", "server_replay.cpp", "quality.cpp", "containers.cpp", "png.cpp"]
HEADERS = ["block_codec.cuh", "block_decode.cuh", "device_io.cuh", "async_copy.cuh", "pdl.cuh", "kernels.h", "batch.h", "host_util.h", "decode.h", "tile_cache.h"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _objects():
    """(object, deps, command) for every translation unit."""
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")]
    jobs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD_DIR, s + ".o")
        cmd = [nvcc, "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
               "-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj]
        jobs.append((obj, [src] + hdrs, cmd))
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD_DIR, s + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall", "-I", CSRC, "-I", INCLUDE,
               "-I", os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj]
        jobs.append((obj, [src] + hdrs, cmd))
    return jobs


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: %s\n%s" % (" ".join(c), out.decode(errors="replace")))


def build(verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    jobs = _objects()
    todo = [cmd for obj, deps, cmd in jobs if _stale(obj, deps)]
    synth_src = os.path.join(CSRC, "synth.c")
    synth_cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-Wall",
                 "-o", SYNTH_LIB, synth_src, "-lm"]
    if _stale(SYNTH_LIB, [synth_src]):
        todo.append(synth_cmd)
    if verbose:
        for c in todo:
            print(" ".join(c))
    _run_parallel(todo)
    objs = [obj for obj, _, _ in jobs]
    if _stale(LIB, objs):
        link = [_nvcc(), "-shared", *ARCH, "-o", LIB, *objs, "-Xcompiler", "-fvisibility=hidden"]
        if verbose:
            print(" ".join(link))
        _run_parallel([link])
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
