"""Known-answer files for the drop-in binary's DEBUG check (TEST INFRASTRUCTURE).

Writes solutions/solution_<DIM>_<ITERATIONS>_<RADIUS>_<DIMENSIONS>d, the raw
float32 grid after ITERATIONS LEGACY sweeps from the reference's initial
state, exactly what the reference's own binary saves before its DEBUG check
(src/main.cu:18-21 -> stencil_cpu, src/stencil_cpu.cu:20-43, saveSolution in
include/stencil_utils.h:38-44).  The grid comes from this package's C
restatement of stencil_cpu, which is bit-identical to the reference's (pinned
by the golden fixtures under tests/golden/).

    python -m oracle.make_solution --dim 64 --dimensions 3 --radius 2 --iterations 8 [--dir .]
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import oracle as O


def solution_name(dim: int, dimensions: int, radius: int, iterations: int) -> str:
    return "solution_%d_%d_%d_%dd" % (dim, iterations, radius, dimensions)


def solution(dim: int, dimensions: int, radius: int, iterations: int, mode: int = O.LEGACY,
             threads: int | None = None) -> np.ndarray:
    """The grid the reference's CPU sweep loop leaves in its first buffer: the
    initial state swept `iterations` times, the second buffer starting at zero
    in LEGACY mode (the reference's calloc'ed h_u2)."""
    shape = (dim,) * dimensions
    u1 = O.init_reference(shape)
    u2 = np.zeros_like(u1) if mode == O.LEGACY else u1.copy()
    return O.run(u1, u2, radius, mode, iterations, threads=threads or O.default_threads())


def write_solution(dim: int, dimensions: int, radius: int, iterations: int, directory: str = ".",
                   mode: int = O.LEGACY) -> str:
    out_dir = os.path.join(directory, "solutions")
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, solution_name(dim, dimensions, radius, iterations))
    grid = np.ascontiguousarray(solution(dim, dimensions, radius, iterations, mode), np.float32)
    with open(path + ".tmp", "wb") as f:
        f.write(grid.tobytes())
    os.replace(path + ".tmp", path)
    return path


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--dim", type=int, required=True)
    ap.add_argument("--dimensions", type=int, default=3)
    ap.add_argument("--radius", type=int, default=1)
    ap.add_argument("--iterations", type=int, default=8)
    ap.add_argument("--jacobi", action="store_true", help="JACOBI mode instead of LEGACY")
    ap.add_argument("--dir", default=".")
    a = ap.parse_args()
    print(write_solution(a.dim, a.dimensions, a.radius, a.iterations, a.dir,
                         O.JACOBI if a.jacobi else O.LEGACY))


if __name__ == "__main__":
    main()
