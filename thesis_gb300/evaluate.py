"""Benchmark harness that writes the reference's results JSON.

Replaces scripts/evaluate_stencils.py (with scripts/evaluate_configuration.sh
and the binary's "ms as the last stdout line" protocol, src/main.cu:89): the
same nested schema

    db[dimension][dim][version_key][radius][iterations][host][config]["time"] = [ms, ...]

with version_key = "<gpus>_gpus_<version>" plus "_unroll_<COARSEN_X>" when the
coarsening factor is above 1, config = "heuristic" or "autotune", one entry per
configuration holding `repeat` sweep-loop times in ms, and the same resume rule
(a configuration whose "time" entry exists is skipped,
scripts/evaluate_stencils.py:186-196), so the thesis' plotting and migration
scripts read GB300 numbers unchanged.

Each configuration runs in-process through the C ABI (stencil_run_host_timed:
upload, ITERATIONS sweeps timed with CUDA events exactly where the reference's
binary times them, download), or with --binary through the drop-in binary
built for that configuration (host/stencil_main.c) by parsing its last stdout
line, as the reference's scripts do.  With --autotune the block shape comes
from results/results_autotune.json (tune_db[dimension][dim][version][radius] =
{"BLOCK_X": .., "BLOCK_Y": .., "BLOCK_Z": ..}, scripts/evaluate_stencils.py:29-37
and :113-117); otherwise the library chooses (the HEURISTIC=1 role).
A configuration the library rejects is stored with an "error" entry instead
of times.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess

import numpy as np

VERSIONS = ["base", "smem", "smem_padded", "smem_register", "coop"]


def version_key(version: str, unroll: int, gpus: int = 1) -> str:
    v = "%d_gpus_%s" % (gpus, version) if gpus > 0 else "_gpu_" + version
    return v + ("_unroll_%d" % unroll if unroll > 1 else "")


def deep_get(d, keys):
    for k in keys:
        if not isinstance(d, dict) or k not in d:
            return None
        d = d[k]
    return d


def load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except FileNotFoundError:
        return {}


def save(path, db):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    with open(path + ".tmp", "w") as f:
        json.dump(db, f)
    os.replace(path + ".tmp", path)


def initial_state(dimensions: int, dim: int) -> np.ndarray:
    """The reference's initial state: outermost layer 1, everything else 0
    (include/stencil_initializer.h:6-52)."""
    u = np.zeros((dim,) * dimensions, np.float32)
    for ax in range(dimensions):
        idx = [slice(None)] * dimensions
        idx[ax] = 0
        u[tuple(idx)] = 1.0
        idx[ax] = dim - 1
        u[tuple(idx)] = 1.0
    return u


def run_inprocess(dimensions, dim, version, radius, iterations, unroll, block, repeat, mode):
    from . import stencil as S
    u = initial_state(dimensions, dim)
    out = np.empty_like(u)
    times = []
    for _ in range(repeat):
        _, _, ms = S.run_host(u, radius, iterations, mode, version, block, unroll, out=out,
                              sweeps_ms=True)
        times.append(float("%.4f" % ms))
    return times


def run_binary(dimensions, dim, version, radius, iterations, unroll, block, repeat, mode):
    from . import build as B
    d = {"DIMENSIONS": dimensions, "DIM": dim, "RADIUS": radius, "ITERATIONS": iterations,
         "COARSEN_X": max(1, unroll), "STENCIL_MODE": mode,
         "SMEM": int(version.startswith("smem")), "PADDED": int(version == "smem_padded"),
         "REGISTER": int(version == "smem_register"), "COOP": int(version == "coop"),
         "HEURISTIC": int(not any(block))}
    if any(block):
        d.update({"BLOCK_X": block[0], "BLOCK_Y": block[1], "BLOCK_Z": block[2]})
    exe = B.build_main(d)
    times = []
    for _ in range(repeat):
        res = subprocess.run([exe], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError((res.stderr or res.stdout).strip().splitlines()[-1])
        times.append(float(res.stdout.strip().splitlines()[-1]))
    return times


def evaluate(dimensions, dims, versions, radii, unrolls, iterations, host="gb300",
             autotune=False, repeat=30, out="results/results_stencils.json",
             tune_path="results/results_autotune.json", binary=False, mode=None, log=print):
    from . import lib as _lib
    mode = _lib.MODE_LEGACY if mode is None else mode
    db = load(out)
    tune_db = load(tune_path) if autotune else {}
    config = "autotune" if autotune else "heuristic"
    run = run_binary if binary else run_inprocess
    for dimension in dimensions:
        for dim in dims:
            for version in versions:
                for unroll in unrolls:
                    v = version_key(version, unroll)
                    v_tune = v[len("1_gpus_"):]
                    for radius in radii:
                        for it in iterations:
                            keys = [str(dimension), str(dim), v, str(radius), str(it), host, config]
                            node = db
                            for k in keys:
                                node = node.setdefault(k, {})
                            if "time" in node or "error" in node:
                                continue
                            block = (0, 0, 0)
                            if autotune:
                                bd = deep_get(tune_db, [str(dimension), str(dim), v_tune, str(radius)])
                                if bd:
                                    block = (int(bd["BLOCK_X"]), int(bd["BLOCK_Y"]),
                                             int(bd.get("BLOCK_Z", 1)) if dimension == 3 else 1)
                            try:
                                node["time"] = run(dimension, dim, version, radius, it, unroll,
                                                   block, repeat, mode)
                            except (_lib.StencilError, RuntimeError) as e:
                                node["error"] = str(e)
                            if log:
                                log("%s: %s" % ("/".join(keys), node.get("time", node.get("error"))))
                            save(out, db)
    save(out, db)
    return db


def main():
    ap = argparse.ArgumentParser(description="write the reference's results JSON for GB300 runs")
    ap.add_argument("--dimensions", type=int, nargs="+", default=[3])
    ap.add_argument("--dims", type=int, nargs="+", default=None,
                    help="grid sides (default: 256 1024 in 3-D, 4096 32768 in 2-D)")
    ap.add_argument("--versions", nargs="+", default=["base", "smem", "smem_padded"], choices=VERSIONS)
    ap.add_argument("--radii", type=int, nargs="+", default=[1, 2, 4, 8, 16])
    ap.add_argument("--unrolls", type=int, nargs="+", default=[1, 2, 4, 8])
    ap.add_argument("--iterations", type=int, nargs="+", default=[8])
    ap.add_argument("--host", default="gb300")
    ap.add_argument("--repeat", type=int, default=30)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--binary", action="store_true",
                    help="run the drop-in binary per configuration and parse its last stdout line")
    ap.add_argument("--jacobi", action="store_true", help="JACOBI mode instead of the reference's update")
    ap.add_argument("--out", default="results/results_stencils.json")
    a = ap.parse_args()
    from . import build, lib as _lib
    build.build()
    for d in a.dimensions:
        dims = a.dims or ([256, 1024] if d == 3 else [4096, 32768])
        evaluate([d], dims, a.versions, a.radii, a.unrolls, a.iterations, a.host, a.autotune,
                 a.repeat, a.out, binary=a.binary,
                 mode=_lib.MODE_JACOBI if a.jacobi else _lib.MODE_LEGACY)


if __name__ == "__main__":
    main()
