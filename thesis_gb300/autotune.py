"""Autotuner for the sweep kernels; replaces the reference's Python-2
Autotuning harness (Autotuning/tuner/*.py driven by
scripts/autotune_configuration.py), which rebuilt and re-ran one binary per
configuration and scored it by the last line of its output.

Here every candidate runs in-process through the C ABI:
  * the search space follows the reference's (block sizes in powers of two
    with 32 <= bx*by*bz <= 1024 and bx >= by >= bz, bx >= 8,
    Autotuning/tuner/optimisation.py:150-160; coarsening factors; radius and
    size from the workload), extended with this library's variants, stream
    tile shapes, cluster sizes and the 2-D temporal blocking depth and tile;
  * the optimiser is a two-level variable tree, as the reference's
    independence tree (Autotuning/tuner/vartree.py): the variant is chosen
    first, each with its default parameters, then the winner's own
    parameters are refined by coordinate descent;
  * a candidate is accepted only if its output is bit-identical to the base
    variant's on a short run (all variants keep the reference summation
    order), and it is scored by the minimum over repeats of CUDA-event time
    per sweep (the reference kept min/median/mean of `repeat` runs,
    Autotuning/tuner/evaluator.py);
  * results go to a JSON database (dims, radius, size bucket) -> choice,
    which load_db() installs into the library (stencil_tuning_set) so that
    STENCIL_VARIANT_AUTO uses it;
  * batches (tune_batch): per class of grid (2-D / 3-D, on a cluster or with
    a whole-GPU launch) the sweeps between halo exchanges, the 3-D temporal
    blocking depth and the 2-D tile, stored in the database's "batch" section
    that Batch(hints_for=batch_hints(db)) applies.
"""
from __future__ import annotations

import argparse
import ctypes
import itertools
import json
import os
import time

from . import lib as _lib

BLOCK_VALUES = [1, 2, 4, 8, 16, 32, 64, 128, 256]


def block_shapes(dims: int):
    """The reference's block filter (Autotuning/tuner/optimisation.py:150-160)."""
    out = []
    for bx, by, bz in itertools.product(BLOCK_VALUES, BLOCK_VALUES, BLOCK_VALUES if dims == 3 else [1]):
        n = bx * by * bz
        if 32 <= n <= 1024 and bx >= by >= bz and bx >= 8:
            out.append((bx, by, bz))
    return out


def variant_space(shape, radius):
    """Variants with their default parameters, then each variant's own
    parameter lists (the second level of the tree)."""
    dims = len(shape)
    nx = shape[-1]
    top = [{"variant": "base"}]
    sub = {"base": {"block": block_shapes(dims), "coarsen_x": [4, 8, 16]}}
    if nx % 4 == 0:
        top.append({"variant": "smem_padded"})
        sub["smem_padded"] = {"block": [b for b in block_shapes(dims) if b[0] <= 64]}
        if dims == 3 and radius <= 4:
            top.append({"variant": "smem_register"})
            # default shape (R <= 2: one row per thread with a 16-slot ring;
            # R >= 3: 16 one-row warps), 64 x 32 tiles, one row per thread
            # with 8 slots, 128 x 16 tiles with two rows per thread and a
            # 16-slot ring (R >= 3), 128 x 32 tiles (R <= 2), and
            # (nx % 128 == 0, nx <= 512) the full-width row-slab kernel
            sub["smem_register"] = {"block": [(0, 0, 0), (16, 32, 1), (0, 1, 0),
                                              (0, 0, 5 if radius <= 2 else 3),
                                              (0, 8, 0), (0, 8, 1)]}
        if radius <= 4:
            top.append({"variant": "cluster"})
            sub["cluster"] = {}
        if dims == 2 and radius <= 4:
            # temporally blocked cooperative engine: sweeps per exchange and
            # the tile (block_x * coarsen_x by block_y cells)
            top.append({"variant": "coop"})
            sub["coop"] = {"temporal": [0, 2, 4, 6, 8, 10, 12, 16, 20],
                           "block": [(0, 0, 1), (16, 16, 1), (24, 20, 1), (32, 16, 1),
                                     (16, 32, 1), (32, 32, 1), (24, 24, 1)]}
        if dims == 3 and radius <= 4:
            # all sweeps in one cooperative launch: one sweep per HBM pass
            # (temporal 0) or, at R <= 2, T sweeps per pass (temporal blocking)
            top.append({"variant": "coop"})
            sub["coop"] = {"temporal": [0, 2, 3, 4] if radius <= 2 else [0]}
    return top, sub


def coordinate_descent(start: dict, space: dict, score, max_rounds: int = 3, min_gain: float = 0.0):
    """Minimises score(config) over the variables of `space`, one variable at
    a time, until a full round changes nothing.  A candidate replaces the
    best so far only when it scores below best * (1 - min_gain) (timing noise
    does not move the choice)."""
    best = dict(start)
    best_s = score(best)
    tried = {json.dumps(best, sort_keys=True): best_s}
    for _ in range(max_rounds):
        changed = False
        for var, values in space.items():
            for v in values:
                cand = dict(best)
                cand[var] = v
                key = json.dumps(cand, sort_keys=True)
                if key not in tried:
                    tried[key] = score(cand)
                if tried[key] < best_s * (1.0 - min_gain):
                    best, best_s, changed = cand, tried[key], True
        if not changed:
            break
    return best, best_s, len(tried)


def optimise(top, sub, score):
    """Two-level tree: best variant at its defaults, then its own parameters."""
    scored = [(score(c), c) for c in top]
    scored.sort(key=lambda t: t[0])
    first_s, first = scored[0]
    space = sub.get(first["variant"], {})
    best, best_s, n = coordinate_descent(first, space, score) if space else (first, first_s, 0)
    return best, best_s, len(top) + n


class GpuEvaluator:
    """Times candidates on the current GPU; rejects any that changes results."""

    def __init__(self, shape, radius, sweeps=20, repeats=3, seed=1):
        import torch
        from . import stencil as S
        self.S, self.torch = S, torch
        self.shape, self.radius, self.sweeps, self.repeats = tuple(shape), radius, sweeps, repeats
        self.u0 = S.init_uniform(self.shape, seed)
        a, b = self.u0.clone(), self.u0.clone()
        self.ref = S.sweep(a, b, radius, 3, _lib.MODE_JACOBI, "base").clone()
        self.a, self.b = self.u0.clone(), self.u0.clone()

    def params(self, cfg):
        return _lib.make_params(self.shape, self.radius, 0, _lib.MODE_JACOBI, cfg["variant"],
                                tuple(cfg.get("block", (0, 0, 0))), cfg.get("coarsen_x", 0),
                                cfg.get("temporal", 0))

    def __call__(self, cfg) -> float:
        S, torch = self.S, self.torch
        try:
            a, b = self.u0.clone(), self.u0.clone()
            out = S.dispatch(self._with_iters(cfg, 3), a, b)
            if not torch.equal(out.view(torch.int32), self.ref.view(torch.int32)):
                return float("inf")
            best = float("inf")
            for _ in range(self.repeats):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                S.dispatch(self._with_iters(cfg, self.sweeps), self.a, self.b)
                e1.record()
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1) / 1e3 / self.sweeps)
            return best
        except _lib.StencilError:
            return float("inf")

    def _with_iters(self, cfg, iters):
        p = self.params(cfg)
        p.iterations = iters
        return p


def tune(shape, radius, sweeps=20, repeats=3, log=print):
    top, sub = variant_space(shape, radius)
    ev = GpuEvaluator(shape, radius, sweeps, repeats)
    t0 = time.time()
    best, best_s, n = optimise(top, sub, ev)
    entry = {"dims": len(shape), "radius": radius, "shape": list(shape),
             "bucket": 1 << (max(shape) - 1).bit_length(), "choice": best,
             "us_per_sweep": best_s * 1e6, "candidates": n, "tune_s": time.time() - t0}
    if log:
        log(json.dumps(entry))
    return entry


def install(entry):
    """Puts one database entry into the library's tuning table."""
    shape = tuple(entry["shape"])
    key = _lib.make_params(shape, entry["radius"], 0)
    c = entry["choice"]
    choice = _lib.make_params(shape, entry["radius"], 0, _lib.MODE_JACOBI, c["variant"],
                              tuple(c.get("block", (0, 0, 0))), c.get("coarsen_x", 0),
                              c.get("temporal", 0))
    _lib.check(_lib.load().stencil_tuning_set(ctypes.byref(key), ctypes.byref(choice)),
               "stencil_tuning_set")


def load_db(path):
    with open(path) as f:
        db = json.load(f)
    for e in db.get("entries", []):
        install(e)
    return db


def save_db(path, entries, device=""):
    db = {"version": 1, "device": device, "entries": entries}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(db, f, indent=1)
    os.replace(tmp, path)


def tune_batch_cluster_size(make_jobs, sizes=(1, 2, 4, 8, 16), log=print):
    """Chooses the cluster size of a batched launch by timing it: make_jobs()
    returns fresh (d_u1, d_u2, radius, iterations, mode) jobs."""
    import torch
    from . import stencil as S
    best, best_t = None, float("inf")
    for c in sizes:
        jobs = make_jobs()
        try:
            bt = S.Batch(jobs, cluster_size=c, engine="phased")
        except _lib.StencilError:
            continue
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        bt.launch()
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        bt.close()
        if log:
            log("cluster_size %d: %.3f s" % (c, t))
        if t < best_t:
            best, best_t = c, t
    return best, best_t


# ---- batches: per-class tuning fields of stencil_batch_job ------------------
#
# The batch engine runs a grid on a thread-block cluster when it fits the
# cluster's shared memory (and, for 3-D, below about 106^3 from L2) and gives
# larger ones a whole-GPU launch.  Each class has its own knobs:
#   2d_small / 3d_small (on clusters): sweeps between halo exchanges in shared
#     memory (temporal: a cap on 8, 4, 2, 1);
#   2d_large (whole GPU): the temporally blocked engine's depth and tile where
#     the grid fits one tile per SM;
#   3d_large (whole GPU): temporal 0 = the one-sweep-per-pass stream kernel,
#     >= 2 = the temporally blocked kernel with that depth (R <= 2).
BATCH_SPACE = {
    "2d_small": {"temporal": [0, 1, 2, 4, 8]},
    "2d_large": {"temporal": [0, 2, 4, 8, 12, 16],
                 "tile": [(0, 0), (32, 16), (64, 16), (32, 32), (64, 32), (128, 16)]},
    "3d_small": {"temporal": [0, 1, 2, 4, 8]},
    "3d_large": {"temporal": [0, 2, 3]},
}


def batch_class(shape) -> str:
    side = max(shape)
    if len(shape) == 2:
        return "2d_small" if side <= 640 else "2d_large"
    return "3d_small" if side <= 106 else "3d_large"


def batch_hints(db):
    """hints_for(shape) for thesis_gb300.stencil.Batch from a database's
    "batch" section ({} when it has none)."""
    table = (db or {}).get("batch", {})

    def hints_for(shape):
        return table.get(batch_class(shape), {}).get("choice")
    return hints_for


def tune_batch(make_jobs, classes=None, repeats=2, log=print):
    """Per-class tuning of a batch: make_jobs(cls) returns fresh (d_u1, d_u2,
    radius, iterations, mode) jobs of that class (a proxy of the batch, e.g.
    some of its grids with fewer sweeps).  Each class's fields are chosen by
    coordinate descent over BATCH_SPACE, scored by the CUDA-event time of one
    batched launch (min over repeats); a candidate whose results differ from
    the library's default choice in any bit is rejected.  Returns
    {class: {"choice": {...}, "s": seconds, "default_s": ...}}."""
    import torch
    from . import stencil as S
    out = {}
    for cls in classes or list(BATCH_SPACE):
        jobs = make_jobs(cls)
        if not jobs:
            continue
        init = [(j[0].clone(), j[1].clone()) for j in jobs]
        ref = None

        def score(cfg):
            nonlocal ref
            hint = {"temporal": cfg.get("temporal", 0), "tile": tuple(cfg.get("tile", (0, 0)))}
            best = float("inf")
            for _ in range(repeats):
                for (u1, u2), job in zip(init, jobs):
                    job[0].copy_(u1)
                    job[1].copy_(u2)
                try:
                    bt = S.Batch([tuple(j[:5]) + (hint,) for j in jobs], engine="phased")
                except _lib.StencilError:
                    return float("inf")
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                bt.launch()
                e1.record()
                e1.synchronize()
                res = [bt.result(k).clone() for k in range(len(jobs))]
                bt.close()
                best = min(best, e0.elapsed_time(e1) / 1e3)
            if ref is None:
                ref = res
            elif any(not torch.equal(x.view(torch.int32), y.view(torch.int32)) for x, y in zip(res, ref)):
                return float("inf")
            return best

        start = {"temporal": 0, "tile": (0, 0)}
        default_s = score(start)  # also records the reference results
        space = {k: v for k, v in BATCH_SPACE[cls].items()}
        best, best_s, n = coordinate_descent(start, space, score)
        out[cls] = {"choice": {"temporal": best.get("temporal", 0), "tile": list(best.get("tile", (0, 0)))},
                    "s": best_s, "default_s": default_s, "candidates": n, "jobs": len(jobs)}
        if log:
            log("batch %s: %s %.4f s (default %.4f s, %d candidates)"
                % (cls, out[cls]["choice"], best_s, default_s, n))
        del jobs, init, ref
        torch.cuda.empty_cache()
    return out


# ---- batches, one-launch engine: CTAs per grid ----------------------------
#
# The one-launch engine gives each grid a team of CTAs (the device's CTA
# count halved repeatedly); its default is the grid's update cells / 50000.
# The tuner picks, per class of grid, the cells per CTA that set each grid's
# team field (cells of the whole grid, border included).
BATCH1_SPACE = {cls: {"cells_per_cta": [12500, 25000, 50000, 100000, 200000]}
                for cls in ("2d_small", "2d_large", "3d_small", "3d_large")}


def team_for(shape, cells_per_cta) -> int:
    """The team field for a grid: its cells / cells_per_cta, at least one CTA
    (the library rounds it down to a team size it has)."""
    n = 1
    for d in shape:
        n *= d
    return max(1, n // int(cells_per_cta))


def batch_team_hints(db):
    """hints_for(shape) -> {"team": ...} for thesis_gb300.stencil.Batch from a
    database's "batch_one_launch" section (None for classes it does not
    cover)."""
    table = (db or {}).get("batch_one_launch", {})

    def hints_for(shape):
        c = table.get(batch_class(shape), {}).get("choice")
        return {"team": team_for(shape, c["cells_per_cta"])} if c else None
    return hints_for


def tune_batch_teams(make_jobs, classes=None, repeats=1, time_batch=None, log=print):
    """Tuning of the one-launch engine's team sizes: make_jobs() returns fresh
    (d_u1, d_u2, radius, iterations, mode) jobs of the whole batch (a proxy,
    e.g. its grids with a tenth of their sweeps: the classes share the GPU
    in one launch, so each is tuned beside the others).  The cells per CTA
    of each class present (BATCH1_SPACE) are chosen by coordinate descent
    from the library's default, each candidate setting every grid's team
    field and scored by the CUDA-event time of one launch (min over
    repeats) and kept only when it gains 1 %; a candidate whose results
    differ in any bit from the default's is rejected.  time_batch(jobs_with_hints) -> (seconds,
    results) replaces the GPU timing (for tests).  Returns {class: {"choice":
    {"cells_per_cta": n}, "s": seconds, "default_s": ...}}."""
    def gpu_time(jobs):
        import torch
        from . import stencil as S
        bt = S.Batch(jobs, engine="one_launch")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        bt.launch()
        e1.record()
        e1.synchronize()
        res = [bt.result(k) for k in range(len(jobs))]
        bt.close()
        return e0.elapsed_time(e1) / 1e3, res

    time_batch = time_batch or gpu_time
    jobs = make_jobs()
    if not jobs:
        return {}
    cls_of = [batch_class(tuple(j[0].shape)) for j in jobs]
    present = [c for c in BATCH1_SPACE if c in set(cls_of) and (classes is None or c in classes)]
    init = [(j[0].clone(), j[1].clone()) for j in jobs]
    ref = None

    def score(cfg):
        nonlocal ref
        best = float("inf")
        for _ in range(repeats):
            for (u1, u2), job in zip(init, jobs):
                job[0].copy_(u1)
                job[1].copy_(u2)
            hinted = [tuple(j[:5]) + ({"team": team_for(tuple(j[0].shape), cfg[c])} if c in cfg else {},)
                      for j, c in zip(jobs, cls_of)]
            try:
                t, res = time_batch(hinted)
            except _lib.StencilError:
                return float("inf")
            if ref is None:
                ref = [x.clone() for x in res]
            elif any(not _bits_equal(x, y) for x, y in zip(res, ref)):
                return float("inf")
            best = min(best, t)
        return best

    start = {c: 50000 for c in present}
    default_s = score(start)  # also records the reference results
    space = {c: list(BATCH1_SPACE[c]["cells_per_cta"]) for c in present}
    # a choice must gain 1 % on the proxy: smaller differences were timing
    # noise on the full batch (GB300: a 3-D choice that gained 1.6 % on one
    # box lost 0.7 % on another)
    best, best_s, n = coordinate_descent(start, space, score, min_gain=0.01)
    out = {c: {"choice": {"cells_per_cta": best[c]}, "s": best_s, "default_s": default_s,
               "candidates": n, "jobs": len(jobs)} for c in present}
    if log:
        log("batch (one launch): %s %.4f s (default %.4f s, %d candidates)"
            % ({c: best[c] for c in present}, best_s, default_s, n))
    return out


def _bits_equal(x, y):
    import torch
    return x.shape == y.shape and torch.equal(x.contiguous().view(torch.int32), y.contiguous().view(torch.int32))


def main():
    ap = argparse.ArgumentParser(description="tune the sweep kernels for one workload")
    ap.add_argument("--shape", type=int, nargs="+", required=True)
    ap.add_argument("--radius", type=int, default=1)
    ap.add_argument("--sweeps", type=int, default=20)
    ap.add_argument("--db", default="tuning.json")
    args = ap.parse_args()
    import torch
    from . import build
    build.build()
    entries = []
    if os.path.exists(args.db):
        entries = json.load(open(args.db)).get("entries", [])
    e = tune(args.shape, args.radius, args.sweeps)
    entries = [x for x in entries if not (x["dims"] == e["dims"] and x["radius"] == e["radius"]
                                          and x["bucket"] == e["bucket"])] + [e]
    save_db(args.db, entries, torch.cuda.get_device_name())


if __name__ == "__main__":
    main()
