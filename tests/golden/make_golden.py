"""Generates the LEGACY golden fixtures from the reference's own CPU path.

Run here, where the reference sources exist:  python tests/golden/make_golden.py

For each configuration it builds the reference's src/stencil_cpu.cu (unchanged,
through oracle/ref_cpu_main.cu, recipe oracle/build.py), runs it, and stores the
raw float32 solution it writes (include/stencil_utils.h:16-44) as a compressed
.npz under tests/golden/, together with the configuration.  The reference
initial state is include/stencil_initializer.h:6-52 and its second buffer is a
fresh malloc (zero pages), i.e. LEGACY semantics with a zero second buffer.
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build  # noqa: E402

# (dims, dim, radius, iterations): the reference's sweep sets use 8 sweeps
# (scripts/evaluate_stencils.py:9) and radii 1..16 (:11); odd counts and
# non-power-of-two sides are added as edge cases.
CONFIGS = [
    (2, 64, 1, 7), (2, 64, 1, 8), (2, 67, 3, 8),
    (2, 256, 1, 8), (2, 256, 2, 8), (2, 256, 4, 8), (2, 256, 8, 8), (2, 256, 16, 8),
    (3, 32, 1, 8), (3, 33, 2, 5), (3, 40, 4, 8), (3, 64, 1, 8), (3, 64, 2, 8),
    (3, 48, 3, 7), (3, 64, 8, 4),
]


def fixture_name(dims, dim, radius, iters):
    return "legacy_%dd_%d_r%d_i%d.npz" % (dims, dim, radius, iters)


def main():
    if not build.reference_available():
        raise SystemExit("reference sources not found")
    exes = build.build_ref(CONFIGS)
    out_dir = os.path.dirname(os.path.abspath(__file__))
    with tempfile.TemporaryDirectory() as tmp:
        for cfg, exe in zip(CONFIGS, exes):
            dims, dim, radius, iters = cfg
            path, secs = build.run_ref(exe, tmp)
            data = np.fromfile(path, dtype=np.float32)
            assert data.size == dim ** dims
            grid = data.reshape((dim,) * dims)
            np.savez_compressed(os.path.join(out_dir, fixture_name(*cfg)), grid=grid,
                                dims=dims, dim=dim, radius=radius, iterations=iters)
            print("%-28s finite=%s max=%g" % (fixture_name(*cfg), np.isfinite(grid).all(),
                                              np.abs(grid).max()))


if __name__ == "__main__":
    main()
