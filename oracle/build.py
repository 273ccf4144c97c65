"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles the C restatement ``stencil_oracle.c`` with gcc
  into ``oracle/liboracle.so`` (works here and on the GPU host).
* ``build_ref(configs)`` compiles the reference's own ``src/stencil_cpu.cu``
  through the wrapper ``ref_cpu_main.cu`` with nvcc, one binary per
  (DIMENSIONS, DIM, RADIUS, ITERATIONS), into ``oracle/_ref/``.  It needs the
  reference sources and is skipped where they are absent.
* ``build_ref_gpu(configs)`` compiles the reference's own one-sweep GPU
  kernels through the wrapper ``ref_gpu_kernels.cu`` into one sm_103a cubin
  per compile-time configuration, into ``oracle/_ref/`` (device code only, so
  the cubins built here run on the GPU host, which has no reference sources).  The reference
  Makefile's own ``stencil_cpu`` target cannot be used: src/stencil_cpu.cpp:1
  includes a header that does not exist and Makefile:72-73 compiles CUDA code
  with gcc.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("STENCIL_REFERENCE_ROOT", "/root/reference")
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "stencil_oracle.c")
    hdr = os.path.join(HERE, "stencil_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-std=c99", "-Wall", "-o", tmp, src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


def reference_available() -> bool:
    return os.path.exists(os.path.join(REF_ROOT, "src", "stencil_cpu.cu"))


def ref_binary(dims: int, dim: int, radius: int, iterations: int) -> str:
    return os.path.join(REF_DIR, "stencil_cpu_%dd_%d_r%d_i%d" % (dims, dim, radius, iterations))


def build_ref(configs, jobs: int = 8) -> list[str]:
    """configs: iterable of (dims, dim, radius, iterations)."""
    if not reference_available():
        return []
    os.makedirs(REF_DIR, exist_ok=True)
    wrapper = os.path.join(HERE, "ref_cpu_main.cu")
    procs, out = [], []
    for dims, dim, radius, iters in configs:
        exe = ref_binary(dims, dim, radius, iters)
        out.append(exe)
        if os.path.exists(exe) and os.path.getmtime(exe) >= os.path.getmtime(wrapper):
            continue
        cmd = ["nvcc", "-O3", "-I", REF_ROOT, "-o", exe, wrapper,
               "-D", "DIMENSIONS=%d" % dims, "-D", "DIM=%d" % dim,
               "-D", "RADIUS=%d" % radius, "-D", "ITERATIONS=%d" % iters]
        procs.append(subprocess.Popen(cmd))
        if len(procs) >= jobs:
            for p in procs:
                if p.wait() != 0:
                    raise RuntimeError("reference CPU build failed")
            procs = []
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference CPU build failed")
    return out


# Reference GPU kernel configurations: (DIMENSIONS, DIM, RADIUS, BLOCK_X,
# BLOCK_Y, BLOCK_Z, COARSEN_X).  Every variant is built for each; the DIM 64
# ones serve the parity tests (golden fixtures), the 512 ones the speed
# comparison.
REF_GPU_SHAPES_512 = [(32, 4, 4, 1), (32, 8, 4, 1), (64, 4, 4, 1), (32, 8, 2, 1), (32, 4, 4, 2),
                      (32, 8, 2, 4)]
# 2-D 256^2 R=1 (the 1000-sweep configuration), and a 64^2 parity case
REF_GPU_SHAPES_256 = [(32, 8, 1, 1), (32, 4, 1, 1), (64, 4, 1, 1), (32, 16, 1, 1), (32, 8, 1, 2),
                      (64, 8, 1, 1), (128, 2, 1, 1)]
REF_GPU_CONFIGS = ([(3, 64, r, 32, 4, 4, 1) for r in (1, 2)] + [(3, 64, 2, 32, 4, 4, 2)] +
                   [(3, 512, r, bx, by, bz, cf) for r in (1, 4) for (bx, by, bz, cf) in REF_GPU_SHAPES_512] +
                   [(2, 64, 1, 32, 8, 1, 1)] +
                   [(2, 256, 1, bx, by, bz, cf) for (bx, by, bz, cf) in REF_GPU_SHAPES_256])


def ref_cubin(cfg) -> str:
    return os.path.join(REF_DIR, "gpu_%dd_%d_r%d_b%dx%dx%d_cf%d.cubin" % tuple(cfg))


def build_ref_gpu(configs=None, jobs: int = 8) -> list[str]:
    """One cubin per configuration.  The variant (base, smem, smem_padded,
    smem_register) is chosen at launch by kernel name, so the SMEM, PADDED and
    REGISTER macros stay at their defaults here."""
    if not reference_available():
        return []
    os.makedirs(REF_DIR, exist_ok=True)
    wrapper = os.path.join(HERE, "ref_gpu_kernels.cu")
    procs, out = [], []
    for cfg in configs or REF_GPU_CONFIGS:
        dims, dim, radius, bx, by, bz, cf = cfg
        cub = ref_cubin(cfg)
        out.append(cub)
        if os.path.exists(cub) and os.path.getmtime(cub) >= os.path.getmtime(wrapper):
            continue
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
               "-I", REF_ROOT, "-o", cub, wrapper,
               "-D", "DIMENSIONS=%d" % dims, "-D", "DIM=%d" % dim, "-D", "RADIUS=%d" % radius,
               "-D", "BLOCK_X=%d" % bx, "-D", "BLOCK_Y=%d" % by, "-D", "BLOCK_Z=%d" % bz,
               "-D", "COARSEN_X=%d" % cf]
        procs.append(subprocess.Popen(cmd))
        if len(procs) >= jobs:
            for p in procs:
                if p.wait() != 0:
                    raise RuntimeError("reference GPU kernel build failed")
            procs = []
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference GPU kernel build failed")
    return out


def run_ref(exe: str, workdir: str) -> tuple[str, float]:
    """Runs one reference binary in workdir; returns (solution path, seconds)."""
    os.makedirs(workdir, exist_ok=True)
    res = subprocess.run([exe], cwd=workdir, capture_output=True, text=True, check=True)
    secs = float("nan")
    for line in res.stdout.splitlines():
        if line.startswith("cpu_stencil:"):
            secs = float(line.split()[1])
    name = None
    for line in res.stdout.splitlines():
        if line.startswith("saving "):
            name = line.split()[1].rstrip(":")
    return os.path.join(workdir, name), secs


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
