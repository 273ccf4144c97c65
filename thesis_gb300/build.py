"""Builds libstencil_gb300.so in-tree with nvcc for sm_103a.

Each ``csrc/*.cu`` is compiled to an object in parallel (relocatable device
code, because the device status word is shared between translation units),
then nvcc device-links and links them into one shared library with the CUDA
runtime linked statically.  The result sits next to this file so that the
library that tests and benchmarks load is the in-tree build.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libstencil_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-rdc=true", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
              "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(d) for d in _deps()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose else []) + \
        ["-c", src, "-o", obj + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, res.stdout, res.stderr))
    if verbose:
        sys.stderr.write(res.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(sources), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), sources))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs + ["-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    return LIB


MAIN_SRC = os.path.join(HERE, "host", "stencil_main.c")
BIN = os.path.join(HERE, "bin")


def main_name(defines: dict) -> str:
    """bin/stencil_<...> named by the configuration's -D values."""
    tag = "_".join("%s%s" % (k.lower(), v) for k, v in sorted(defines.items()))
    return os.path.join(BIN, "stencil_" + (tag or "default"))


def build_main(defines: dict | None = None, out: str | None = None) -> str:
    """Compiles the drop-in stencil binary (host/stencil_main.c) for one
    compile-time configuration, given as the reference's -D macros (DIM,
    DIMENSIONS, RADIUS, ITERATIONS, SMEM, PADDED, REGISTER, COOP, BLOCK_X, ...),
    and links it to the in-tree library (gcc only: the binary calls the C ABI
    and needs no CUDA headers or libraries of its own)."""
    defines = dict(defines or {})
    build()
    out = out or main_name(defines)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = (["gcc", "-O2", "-std=c99", "-Wall", "-I", INCLUDE] +
           ["-D%s=%s" % (k, v) for k, v in sorted(defines.items())] +
           [MAIN_SRC, "-o", out + ".tmp", "-L", HERE, "-lstencil_gb300",
            "-Wl,-rpath," + HERE, "-lm"])
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("stencil_main build failed:\n%s%s" % (res.stdout, res.stderr))
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
