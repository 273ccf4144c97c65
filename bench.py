"""Benchmark of the star-stencil sweep loop on one GB300 (or N replicas).

Workload (one "step"): plain FP32 3-D star stencil, 512^3 grid, radius 1
(7-point), Jacobi update (mean of the 6R axis neighbours), 1000 sweeps,
border and interior i.i.d. uniform [0,1) from a seed.  The same loop at
radius 4 (25-point) is reported as a second line item.  Metric: GCell-updates/s
= (N - 2R)^3 * sweeps / seconds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the CPU restatement of the reference's sweep loop
(the oracle, OpenMP over all host threads) on a bounded sample of the same
workload: the reference's stencil_cpu itself is x86-built from its sources
and does not exist on the GPU host.

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path is a single-GPU solver: no collective); ``value`` sums the cell
updates of all ranks over the slowest rank's time.  The other workloads
(``configs``: 2-D 256^2, the 768^3 refinement, the 512-grid batch, the learned
warm start) and the CPU baseline are N = 1 line items.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIM = 512
SWEEPS = 1000
SEED = 20251203
HBM_BYTES_PER_UPDATE = 8  # one FP32 read + one FP32 write per cell update


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dim", type=int, default=DIM)
    ap.add_argument("--sweeps", type=int, default=SWEEPS)
    ap.add_argument("--radius", type=int, default=1)
    ap.add_argument("--variant", default="auto")
    ap.add_argument("--no-r4", action="store_true", help="skip the radius-4 line item")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 2-D, precision and batching line items")
    ap.add_argument("--profile-case", default=None, metavar="NAME",
                    help="run one small, self-contained case of a hot kernel for a profiler "
                         "(see PROFILE_CASES) and exit")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-warm-start workload (about 4 minutes: data, "
                         "training, 5 x 256 timed solves)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device):
    """The largest of every rank's x (a time in seconds): the replicas' step
    time is the slowest replica's.  Needs the process group when world > 1."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(updates_per_step, steps, world, seconds):
    """Whole-job GCell-updates/s of `world` replicas that each ran `steps`
    steps of `updates_per_step` updates in `seconds` (the max over ranks)."""
    return updates_per_step * steps * world / seconds / 1e9


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(key):
    """DRAM bytes per launch from the committed ncu summary (profiles/traffic.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(key)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", "stencil_clocks_%d_%d.csv" % (os.getpid(), gpu_index))

    def __enter__(self):
        try:
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.out.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except OSError:
            pass
        try:
            os.unlink(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def bench_config(args, world):
    """The workload both arms report (the same dict in the reference arm's line)."""
    return {"workload": "3D %d^3 FP32 star stencil R=%d, Jacobi, %d sweeps per step"
                        % (args.dim, args.radius, args.sweeps),
            "dims": 3, "dim": args.dim, "radius": args.radius, "sweeps": args.sweeps,
            "variant": args.variant, "parallelism": "replicas" if world > 1 else "single",
            "l2": "no flush: 2 x %d MiB working set > 129 MB L2" % (args.dim ** 3 * 4 // 2 ** 20)}


def updates(dim, radius, sweeps):
    return float(dim - 2 * radius) ** 3 * sweeps


def time_device_loop(S, torch, u0, radius, sweeps, variant, steps, warmup, stream):
    """Device-resident timing: inputs already in HBM.  Returns (seconds per step list,
    launches per step)."""
    from thesis_gb300 import lib
    a = u0.clone()
    b = u0.clone()
    p = lib.make_params(tuple(u0.shape), radius, sweeps, lib.MODE_JACOBI, variant)
    L = lib.load()
    res = ctypes.c_void_p()

    def step():
        # each step restarts from the initial state (same work every step)
        a.copy_(u0)
        lib.check(L.stencil_dispatch_ex(ctypes.byref(p), ctypes.c_void_p(a.data_ptr()),
                                        ctypes.c_void_p(b.data_ptr()),
                                        ctypes.c_void_p(stream.cuda_stream), ctypes.byref(res)),
                  "stencil_dispatch_ex")

    with torch.cuda.stream(stream):
        b.copy_(u0)
        for _ in range(warmup):
            step()
        stream.synchronize()
        times = []
        for _ in range(steps):
            # the restart copy is outside the event pair: only the sweeps are timed
            a.copy_(u0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lib.check(L.stencil_dispatch_ex(ctypes.byref(p), ctypes.c_void_p(a.data_ptr()),
                                            ctypes.c_void_p(b.data_ptr()),
                                            ctypes.c_void_p(stream.cuda_stream),
                                            ctypes.byref(res)), "stencil_dispatch_ex")
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    del a, b
    return times


def run_ours(args):
    import torch
    import torch.distributed as dist
    from thesis_gb300 import lib, stencil as S
    from thesis_gb300 import build as B

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if rank == 0 or world == 1:
        B.build()
    if world > 1:
        dist.barrier()
    lib.load()
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)
    shape = (args.dim,) * 3
    u0 = S.init_uniform(shape, SEED, device=dev)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def maxed(x):
        return max_over_ranks(x, world, dev)

    # ---- headline: device-resident sweeps (radius args.radius) ------------
    barrier()
    with ClockSampler(local) as clk:
        barrier()
        step_times = time_device_loop(S, torch, u0, args.radius, args.sweeps, args.variant,
                                      args.steps, args.warmup, stream)
        barrier()
    total = maxed(sum(step_times))
    engine, launches_per_step = S.last_dispatch()
    ups = updates(args.dim, args.radius, args.sweeps)
    value = aggregate_rate(ups, args.steps, world, total)
    # time per sweep (a sweep is one launch, or one grid-barrier phase of the
    # persistent launch; bytes per launch / launch time is the same ratio)
    per_sweep = min(step_times) / args.sweeps
    peak, peak_kind = peaks()
    achieved = ups / args.sweeps * HBM_BYTES_PER_UPDATE / per_sweep / 1e9
    traffic = profile_traffic("stream3d_r%d_512" % args.radius)

    out = {
        "metric": "GCell-updates/s (3D 512^3 FP32 star stencil, Jacobi, 1000 sweeps)",
        "value": round(value, 3),
        "unit": "GCell-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: border and interior i.i.d. uniform [0,1) (SplitMix64, seed %d)" % SEED,
        "config": bench_config(args, world),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_kind": peak_kind, "traffic": traffic,
                     "bytes_per_update": HBM_BYTES_PER_UPDATE,
                     "kernel_us_per_sweep": round(per_sweep * 1e6, 2), "engine": engine},
        "gpu_launches": args.steps * launches_per_step,
    }

    # ---- radius-4 line item ---------------------------------------------
    if not args.no_r4 and args.radius != 4:
        barrier()
        t4 = time_device_loop(S, torch, u0, 4, args.sweeps, args.variant,
                              max(2, args.steps // 2), 2, stream)
        t4s = maxed(sum(t4))
        ups4 = updates(args.dim, 4, args.sweeps)
        per4 = min(t4) / args.sweeps
        ach4 = ups4 / args.sweeps * HBM_BYTES_PER_UPDATE / per4 / 1e9
        out["r4"] = {"value": round(aggregate_rate(ups4, len(t4), world, t4s), 3),
                     "unit": "GCell-updates/s", "ms_per_step": round(t4s / len(t4) * 1e3, 3),
                     "roofline": {"bound": "hbm", "achieved": round(ach4, 1), "peak": peak,
                                  "unit": "GB/s", "frac": round(ach4 / peak, 4),
                                  "traffic": profile_traffic("stream3d_r4_512")}}

    # ---- end to end through the C ABI with host buffers --------------------
    if not args.no_e2e:
        h_in = u0.cpu().pin_memory()
        h_out = torch.empty_like(h_in).pin_memory()
        p = lib.make_params(shape, args.radius, args.sweeps, lib.MODE_JACOBI, args.variant)
        L = lib.load()
        ms = ctypes.c_float()

        def e2e_step():
            lib.check(L.stencil_run_host(ctypes.byref(p), ctypes.c_void_p(h_in.data_ptr()),
                                         ctypes.c_void_p(h_out.data_ptr()), ctypes.byref(ms)),
                      "stencil_run_host")

        for _ in range(max(1, args.warmup - 1)):
            e2e_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        barrier()
        te = maxed(time.perf_counter() - t0)
        nbytes = h_in.numel() * 4
        out["e2e"] = {"value": round(aggregate_rate(ups, args.steps, world, te), 3),
                      "unit": "GCell-updates/s", "h2d_bytes_per_step": nbytes,
                      "d2h_bytes_per_step": nbytes,
                      "api": "stencil_run_host (pinned host in/out, upload + sweeps + download)"}
        L.stencil_release()

    out["clocks"] = clk.summary()

    # ---- the other workloads, each as its own line item (N = 1 only: under
    # torchrun the line measures the replicated headline, and the other ranks
    # would hold their GPUs idle meanwhile) -----------------------------------
    if not args.no_configs and world == 1:
        out["configs"] = {}
        out["configs"]["c1_2d_256"] = bench_c1(S, lib, torch)
        out["configs"]["c3_precision_768"] = bench_c3(S, lib, torch)
        out["configs"]["c4_batch_512"] = bench_c4(S, lib, torch)
        if not args.no_learned:
            from thesis_gb300 import warmstart as W
            seeds = list(range(10_000_000, 10_000_256))
            out["configs"]["c5_learned_512"] = bench_c5(W, torch, seeds)

    # ---- CPU baseline: the oracle on the host cores, bounded sample (N = 1) --
    if not args.no_cpu and world == 1:
        def gpu_sweeps(k):
            a, b = u0.clone(), u0.clone()
            res = S.sweep(a, b, args.radius, k, lib.MODE_JACOBI, args.variant)
            return res.cpu().numpy()

        cb = cpu_baseline(u0.cpu().numpy(), args.radius, target_s=10.0, gpu_sweeps=gpu_sweeps)
        out["fp64_error"] = cb.pop("check")
        out["cpu_baseline"] = cb

    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def bench_c1(S, lib, torch, steps=5):
    """2-D 256^2 R=1, 1000 Jacobi sweeps: the whole loop in one cooperative
    launch over every SM (one tile per CTA, several sweeps per exchange)."""
    shape, R, sweeps = (256, 256), 1, 1000
    u0 = S.init_uniform(shape, SEED)
    a, b = u0.clone(), u0.clone()
    for _ in range(3):
        S.sweep(a, b, R, sweeps, lib.MODE_JACOBI, "auto")
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        a.copy_(u0)
        e0, e1 = _events(torch)
        e0.record()
        S.sweep(a, b, R, sweeps, lib.MODE_JACOBI, "auto")
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    engine, launches = S.last_dispatch()
    ups = 254.0 * 254.0 * sweeps
    import numpy as np
    from oracle import oracle as O
    h = u0.cpu().numpy()
    t0 = time.perf_counter()
    O.run(h.copy(), h.copy(), R, O.JACOBI, sweeps, 1)
    cpu_s = time.perf_counter() - t0
    return {"workload": "2D 256^2 FP32 R=1 Jacobi, 1000 sweeps (one cooperative launch, tiles and "
                        "halos in shared memory, exchanged through L2 every few sweeps)",
            "value": round(ups / min(times) / 1e9, 3), "unit": "GCell-updates/s",
            "ms_per_solve": round(min(times) * 1e3, 4), "us_per_sweep": round(min(times) / sweeps * 1e6, 3),
            "engine": engine, "gpu_launches": launches,
            "bound": "latency (CTA barrier per sweep, L2 round trip per exchange); 512 KiB working set is on-chip",
            "cpu_baseline": {"value": round(ups / cpu_s / 1e9, 3), "unit": "GCell-updates/s",
                             "cores": 1, "kind": "port",
                             "sample": "full workload, oracle single-threaded like stencil_cpu"}}


def bench_c3(S, lib, torch):
    """3-D 768^3 R=4, 2000 sweeps: FP32 loop vs mixed-precision refinement."""
    shape, R, sweeps = (768, 768, 768), 4, 2000
    ups = 760.0 ** 3 * sweeps
    u0 = S.init_fourier(shape, SEED, R, modes=8)
    res = {"workload": "3D 768^3 R=4, 2000 sweeps; Fourier border (8 modes) + uniform interior",
           "unit": "GCell-updates/s"}
    a, b = u0.clone(), u0.clone()
    S.sweep(a, b, R, 20, lib.MODE_JACOBI, "auto")
    a.copy_(u0)
    e0, e1 = _events(torch)
    e0.record()
    fp32 = S.sweep(a, b, R, sweeps, lib.MODE_JACOBI, "auto")
    e1.record()
    e1.synchronize()
    t32 = e0.elapsed_time(e1) / 1e3
    res["fp32"] = {"value": round(ups / t32 / 1e9, 2), "s": round(t32, 3),
                   "rel_residual": S.residual(fp32, R),
                   "roofline_frac": round(ups / t32 * 8 / 1e9 / peaks()[0], 4)}
    fp32 = fp32.clone()
    del a, b
    ws = None
    for st in ("bf16", "fp16"):
        u = u0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        done, outer, rel = S.ir_solve(u, R, sweeps, st, inner_sweeps=50)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        err = float((u - fp32).abs().max() / fp32.abs().max())
        res["ir_" + st] = {"value": round(ups / t / 1e9, 2), "s": round(t, 3), "rel_residual": rel,
                           "normwise_err_vs_fp32": err, "speedup_vs_fp32": round(t32 / t, 3),
                           "bytes_per_update": 6}
        del u
    torch.cuda.empty_cache()
    return res


def c4_jobs(seed=20251204):
    """384 2-D R=1 grids (side log-uniform [64, 2048]) and 128 3-D R=2 grids
    (side log-uniform [32, 256]), sweeps uniform [100, 5000]; sides rounded to
    the nearest integer (about three in four are not multiples of 4: the batch
    sweeps those in pitched copies)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(384):
        s = int(round(np.exp(rng.uniform(np.log(64), np.log(2048)))))
        specs.append(((s, s), 1, int(rng.integers(100, 5001))))
    for _ in range(128):
        s = int(round(np.exp(rng.uniform(np.log(32), np.log(256)))))
        specs.append(((s, s, s), 2, int(rng.integers(100, 5001))))
    return specs


def bench_c4(S, lib, torch):
    """512 grids of uneven sizes and sweep counts.  The line item: the
    one-launch engine -- every grid in ONE cooperative launch, teams of CTAs
    taking grids from device queues -- with the team sizes the autotuner
    picks per class of grid on a proxy, kept when they beat the default plan
    on the batch itself, replayed as a CUDA graph (both plans are reported).
    Beside it
    the phased engine (a persistent cluster launch over a device work queue
    for the grids a cluster sweeps, then persistent whole-GPU launches in
    lanes), with its cluster size and per-class hints picked by the
    autotuner."""
    from thesis_gb300 import autotune as A
    specs = c4_jobs()
    ups = 0.0
    for shape, R, it in specs:
        n = 1.0
        for d in shape:
            n *= d - 2 * R
        ups += n * it
    grids = []
    for k, (shape, R, it) in enumerate(specs):
        u = S.init_uniform(shape, SEED + k)
        grids.append((u, u.clone()))

    def timed(bt, reps=3):
        stream = torch.cuda.Stream()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            bt.launch(stream=stream)  # warm-up
            stream.synchronize()
            with torch.cuda.graph(graph, stream=stream):
                bt.launch(stream=stream)
        times = []
        with torch.cuda.stream(stream):
            for _ in range(reps):
                e0, e1 = _events(torch)
                e0.record(stream)
                graph.replay()  # replays on the current stream
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1) / 1e3)
        del graph
        return min(times)

    jobs = [(g[0], g[1], sp[1], sp[2], lib.MODE_JACOBI) for g, sp in zip(grids, specs)]

    def class_jobs(cls):
        # up to 6 grids of the class with a tenth of their sweeps: the proxy
        # the tuners time (fresh copies, so the benchmark grids stay as made)
        ks = [k for k, sp in enumerate(specs) if A.batch_class(sp[0]) == cls][:6]
        return [(grids[k][0].clone(), grids[k][1].clone(), specs[k][1],
                 max(10, specs[k][2] // 10), lib.MODE_JACOBI) for k in ks]

    # the one-launch engine with its default team sizes, and with the team
    # sizes the autotuner picks per class on a proxy of the batch; the line
    # item keeps the tuner's plan only when it is faster on the batch itself
    # (the proxy has a tenth of the sweeps and misjudged the large 3-D grids
    # on some boxes)
    b1 = S.Batch(jobs, engine="one_launch")
    t1_default = timed(b1)
    launches_d, teams_d = b1.kernel_launches(), b1.teams()
    b1.close()

    def proxy_jobs():
        # every grid with a tenth of its sweeps: the proxy the team tuner
        # times (the classes share the GPU in one launch)
        return [(g[0].clone(), g[1].clone(), sp[1], max(10, sp[2] // 10), lib.MODE_JACOBI)
                for g, sp in zip(grids, specs)]

    teams_tuned = A.tune_batch_teams(proxy_jobs, log=None)
    b1 = S.Batch(jobs, engine="one_launch", hints_for=A.batch_team_hints({"batch_one_launch": teams_tuned}))
    t1_tuned = timed(b1)
    launches_t, teams_t = b1.kernel_launches(), b1.teams()
    b1.close()
    use_tuned = t1_tuned < t1_default
    t1, launches1, teams = (t1_tuned, launches_t, teams_t) if use_tuned else (t1_default, launches_d, teams_d)

    def sample_jobs():
        # every 8th grid, sweeps / 10: a proxy of the batch for the tuner
        return [(grids[k][0], grids[k][1], specs[k][1], max(10, specs[k][2] // 10), lib.MODE_JACOBI)
                for k in range(0, len(specs), 8)]

    csize, _ = A.tune_batch_cluster_size(sample_jobs, log=None)
    tuned = A.tune_batch(class_jobs, log=None)
    bt = S.Batch(jobs, cluster_size=csize, hints_for=A.batch_hints({"batch": tuned}), engine="phased")
    tp = timed(bt)
    cluster_jobs, whole_gpu_jobs = bt.plan()
    launches = bt.kernel_launches()
    bt.close()
    mem = sum(g[0].numel() * 8 for g in grids)
    del grids, jobs
    torch.cuda.empty_cache()
    ragged = sum(1 for shape, _, _ in specs if shape[-1] % 4)
    return {"workload": "512 grids: 384 2D R=1 side 64..2048 + 128 3D R=2 side 32..256, 100..5000 sweeps",
            "ragged_jobs": ragged,
            "value": round(ups / t1 / 1e9, 2), "unit": "GCell-updates/s",
            "s_per_batch": round(t1, 3), "cell_updates": ups, "engine": "one_launch",
            "device_bytes": mem, "graph_replays_per_batch": 1, "kernel_launches_per_batch": launches1,
            "teams": [{"team_ctas": t, "jobs": n} for t, n in teams], "graph": True,
            "team_plan": "tuned" if use_tuned else "default",
            "tuned_teams": {"value": round(ups / t1_tuned / 1e9, 2), "s_per_batch": round(t1_tuned, 3),
                            "cells_per_cta": {c: r["choice"]["cells_per_cta"] for c, r in teams_tuned.items()}},
            "default_teams": {"value": round(ups / t1_default / 1e9, 2), "s_per_batch": round(t1_default, 3)},
            "roofline_frac_if_hbm": round(ups / t1 * 8 / 1e9 / peaks()[0], 4),
            "phased": {"value": round(ups / tp / 1e9, 2), "s_per_batch": round(tp, 3),
                       "kernel_launches_per_batch": launches, "cluster_jobs": cluster_jobs,
                       "whole_gpu_jobs": whole_gpu_jobs, "cluster_size": csize,
                       "tuned": {c: r["choice"] for c, r in tuned.items()}}}


def bench_c5(W, torch, seeds):
    """2-D Laplace 512^2 to relative residual 1e-5 on 256 held-out seeds:
    the learned warm start followed by the FP16 mixed-precision refinement
    against plain FP32 Jacobi from zero on the same GPU (the library's best
    plain engine for the grid), every solve timed with CUDA events around
    all of its GPU work, one problem at a time."""
    from thesis_gb300.unet import UNet
    t0 = time.time()
    fields, sols = W.generate_pairs(20000, 128, sweeps=40000)
    gen_s = time.time() - t0
    net = UNet(seed=0)
    losses, train_s = W.train(net, fields, sols, epochs=40, batch=64, lr=1e-3)
    del fields, sols
    torch.cuda.empty_cache()
    arms = ["zero_fp32", "learned_ir_fp16", "learned_fp32", "learned_ir_bf16", "zero_ir_fp16"]
    res = W.evaluate(net, seeds, 512, 1e-5, arms=arms, n_exact=8, log=lambda *a: None)
    head, plain = res["learned_ir_fp16"], res["zero_fp32"]
    return {"workload": "2D Laplace 512^2, 5-point Jacobi to relative residual 1e-5, 256 held-out "
                        "seeds; U-Net (4 levels, 32 base channels, BF16 weights) trained on 20k "
                        "128^2 Jacobi-generated pairs",
            "metric": "time to tolerance per solve, learned warm start + FP16 refinement vs plain "
                      "FP32 Jacobi from zero",
            "speedup_vs_plain": round(head["speedup_vs_plain"], 3),
            "time_to_tol_s": round(head["time_per_solve_s"], 6),
            "plain_time_to_tol_s": round(plain["time_per_solve_s"], 6),
            "sweeps": head["mean_sweeps"], "plain_sweeps": plain["mean_sweeps"],
            "fp64_normwise_err": head["fp64_normwise_err_max"],
            "plain_fp64_normwise_err": plain["fp64_normwise_err_max"],
            "arms": {a: res[a] for a in arms},
            "check_every_plain": res["check_every_plain"], "ir_inner_sweeps": res["ir_inner_sweeps"],
            "timing": res["timing"], "pairs": 20000, "gen_s": round(gen_s, 1),
            "train_s": round(train_s, 1), "final_loss": losses[-1]}


def cpu_baseline(host_grid, radius, target_s=10.0, threads=None, gpu_sweeps=None, check_sweeps=100):
    """Times the oracle's FP32 sweep (CPU restatement of src/stencil_cpu.cu) on
    the host cores for about target_s seconds of sweeps over the full grid.
    The same leg checks the GPU against it: gpu_sweeps(k) returns the GPU's
    grid after k sweeps of the workload, compared with the FP32 oracle (bit
    for bit: same summation order) and the FP64 oracle (normwise error) after
    check_sweeps sweeps; returned under "check"."""
    import numpy as np
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    a = np.ascontiguousarray(host_grid, np.float32).copy()
    b = a.copy()
    dim = a.shape[0]
    t0 = time.perf_counter()
    O.sweep(a, b, radius, O.JACOBI, threads)  # one sweep to size the sample
    one = time.perf_counter() - t0
    n = max(1, int(target_s / max(one, 1e-6)))
    t0 = time.perf_counter()
    O.run(a, b, radius, O.JACOBI, n, threads)
    dt = time.perf_counter() - t0
    out = {"value": round(updates(dim, radius, n) / dt / 1e9, 4), "unit": "GCell-updates/s",
           "cores": threads, "kind": "port",
           "sample": "%d sweeps of %d^3 R=%d Jacobi (oracle, OpenMP %d threads, %.1f s)"
                     % (n, dim, radius, threads, dt)}
    del a, b
    if gpu_sweeps is not None:
        got = gpu_sweeps(check_sweeps)
        h = np.ascontiguousarray(host_grid, np.float32)
        want = O.run(h.copy(), h.copy(), radius, O.JACOBI, check_sweeps, threads)
        exact = bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))
        del want
        h64 = h.astype(np.float64)
        r64 = O.run(h64.copy(), h64.copy(), radius, O.JACOBI, check_sweeps, threads)
        err = float(np.abs(got - r64).max() / np.abs(r64).max())
        out["check"] = {"sweeps": check_sweeps, "normwise_vs_fp64_oracle": err,
                        "bit_exact_vs_fp32_oracle": exact,
                        "what": "GPU grid after %d sweeps of the benchmark workload against the "
                                "oracle's FP32 and FP64 runs of the same sweeps (the 1000-sweep "
                                "bit-exact comparison is tests/test_full_iteration_gpu.py)"
                                % check_sweeps}
    return out


def run_reference(args):
    """The reference arm: the reference's CPU sweep loop (src/stencil_cpu.cu:20-43)
    timed on the host cores on the same workload.  The reference's own
    stencil_cpu is built from its sources only where they are present (not on
    the GPU host), so its bit-identical restatement (the oracle, OpenMP over
    all host threads) stands in for it.  Each step times a bounded sample of
    the 1000-sweep workload: `sampled_sweeps_per_step` full-grid sweeps, and
    `value` is GCell-updates/s over those sweeps."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    shape = (args.dim,) * 3
    u = O.uniform(shape, SEED)
    threads = os.cpu_count() or 1
    a, b = u.copy(), u.copy()
    t0 = time.perf_counter()
    O.sweep(a, b, args.radius, O.JACOBI, threads)
    one = time.perf_counter() - t0
    per_step = max(1, int(8.0 / max(one, 1e-6)))
    for _ in range(args.warmup):
        O.sweep(a, b, args.radius, O.JACOBI, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.run(a, b, args.radius, O.JACOBI, per_step, threads)
    dt = time.perf_counter() - t0
    value = updates(args.dim, args.radius, per_step) * args.steps / dt / 1e9
    sample = ("%d of the %d sweeps per step, full %d^3 grid R=%d (oracle restatement of "
              "src/stencil_cpu.cu, bit-identical to it, OpenMP %d threads; the reference's "
              "stencil_cpu is single-threaded and is not built on the GPU host)"
              % (per_step, args.sweeps, args.dim, args.radius, threads))
    out = {
        "impl": "reference",
        "metric": "GCell-updates/s (3D 512^3 FP32 star stencil, Jacobi, 1000 sweeps)",
        "value": round(value, 4),
        "unit": "GCell-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3),
        "sampled_sweeps_per_step": per_step,
        "ms_per_step_extrapolated_to_full_step": round(dt / args.steps * args.sweeps / per_step * 1e3, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: border and interior i.i.d. uniform [0,1) (SplitMix64, seed %d)" % SEED,
        "config": bench_config(args, world),
        "cpu_baseline": {"value": round(value, 4), "unit": "GCell-updates/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "GCell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def _profile_case(case):
    """Small, self-contained runs of each hot kernel for a profiler: each case
    warms up, then runs the kernel a few more times.  Where the kernel is
    HBM-bound the working set exceeds the 129 MB L2, yet a full ncu capture of
    one launch ends in seconds (a few hundred MB on the device at most)."""
    import torch
    from thesis_gb300 import build, lib, stencil as S
    build.build()
    J = lib.MODE_JACOBI

    def cube(n, seed=1):
        u = S.init_uniform((n, n, n), seed)
        return u.clone(), u.clone()

    if case in ("stream_r1", "stream_r4", "stream_r1_512", "stream_r4_512"):
        # one launch per sweep of the stream kernel
        R = 1 if case.startswith("stream_r1") else 4
        a, b = cube(512 if case.endswith("_512") else 320)
        for _ in range(4):
            S.sweep(a, b, R, 2, J, "smem_register")
    elif case in ("persist_r1_512", "persist_r4_512"):
        # the persistent engine AUTO runs: 8 sweeps in one cooperative launch
        a, b = cube(512)
        for _ in range(3):
            S.sweep(a, b, 1 if case == "persist_r1_512" else 4, 8, J, "coop", temporal=1)
    elif case in ("tb_r1_t2", "tb_r1_t3", "tb_r1_t4"):
        # 3-D temporal blocking, T sweeps per HBM pass, one pass per launch
        T = int(case[-1])
        a, b = cube(320)
        for _ in range(4):
            S.sweep(a, b, 1, T, J, "coop", temporal=T)
    elif case in ("base_r1", "tile_r1", "rows3d_r1"):
        # base: float4 chunks through L1/L2; tile: TMA box tile with halo
        # (smem / smem_padded roles); rows3d: full-width row slabs by bulk copy
        a, b = cube(512 if case == "rows3d_r1" else 320)
        variant, block = {"base_r1": ("base", (0, 0, 0)), "tile_r1": ("smem_padded", (0, 0, 0)),
                          "rows3d_r1": ("smem_register", (0, 8, 1))}[case]
        for _ in range(4):
            S.sweep(a, b, 1, 2, J, variant, block=block)
    elif case == "rows2d_8192":
        # the persistent 2-D rows engine (grid barrier per sweep), 256 MB per buffer
        u = S.init_uniform((8192, 8192), 1)
        a, b = u.clone(), u.clone()
        for _ in range(3):
            S.sweep(a, b, 1, 8, J, "coop")
    elif case == "cluster_2d256":
        u = S.init_uniform((256, 256), 1)
        a, b = u.clone(), u.clone()
        for _ in range(4):
            S.sweep(a, b, 1, 1000, J, "cluster")
    elif case == "tb2d_256":
        # the 2-D temporally blocked engine AUTO runs on 256^2, 1000 sweeps per launch
        u = S.init_uniform((256, 256), 1)
        a, b = u.clone(), u.clone()
        for _ in range(4):
            S.sweep(a, b, 1, 1000, J, "auto")
    elif case == "ir2d_512":
        # the persistent 2-D refinement engine: outer steps of 500 FP16 correction
        # sweeps on the 512^2 Laplace problem
        u = S.init_laplace2d((512, 512), 3)
        ws = S.ir_workspace((512, 512), 1, "fp16")
        for _ in range(3):
            S.ir_solve_ex(u, 1, 1000, "fp16", inner_sweeps=500, workspace=ws)
    elif case in ("ir_r1", "ir_r2", "ir_r4"):
        # mixed-precision refinement, 512^3, 100 sweeps in outer steps of 50
        R = int(case[-1])
        u = S.init_fourier((512, 512, 512), 1, R)
        for _ in range(2):
            S.ir_solve(u, R, 100, "bf16", inner_sweeps=50)
    elif case == "lp_sweep_r4":
        u = S.init_fourier((384, 384, 384), 1, 4)
        for _ in range(2):
            S.ir_solve(u, 4, 8, "bf16", inner_sweeps=8)
    elif case in ("conv_tc", "conv_mma"):
        # one U-Net layer shape (d2a: 32^2, 384 -> 128 channels, batch 64) on each engine
        from thesis_gb300 import unet as U
        L = U._L()
        x = torch.randn(64, 32, 32, 384, device="cuda").to(torch.bfloat16)
        w = (torch.randn(128, 9, 384, device="cuda") * 0.05).to(torch.bfloat16)
        bias = torch.zeros(128, device="cuda")
        y = torch.empty(64, 32, 32, 128, dtype=torch.bfloat16, device="cuda")
        eng = 1 if case == "conv_tc" else 2
        for _ in range(4):
            U._chk(L.unet_conv3x3_fwd_engine(ctypes.byref(U.view(x)), U._p(w), U._p(bias),
                                             ctypes.byref(U.view(y)), 1, 1, eng, None), case)
    elif case == "unet_train":
        from thesis_gb300 import warmstart as W
        from thesis_gb300.unet import UNet
        fields = W.borders(range(64), 128)
        target = W.coons_fill(fields)
        net = UNet(seed=0)
        for _ in range(3):
            net.zero_grad()
            B = net.loss_and_grad(fields, target)
            net.backward(B)
            net.adam_step()
    elif case == "batch_small":
        jobs = []
        for k in range(64):
            n = 64 + 32 * (k % 8)
            u = S.init_uniform((n, n), k)
            jobs.append((u, u.clone(), 1, 200 + 10 * k, J))
        bt = S.Batch(jobs, engine="phased")
        for _ in range(3):
            bt.launch()
    elif case == "batch_3d_small":
        # the cluster phase of the benchmark batch's small 3-D part: 18 grids
        # of 56^3 .. 104^3, R = 2, 100 sweeps each, swept from L2 by clusters
        sides = [56 + 8 * (k % 7) for k in range(18)]
        jobs = []
        for k, n in enumerate(sides):
            u = S.init_uniform((n, n, n), k)
            jobs.append((u, u.clone(), 2, 100, J))
        bt = S.Batch(jobs, engine="phased")
        for _ in range(3):
            bt.launch()
        cells = sum((n - 4) ** 3 * 100 for n in sides)
        best = 1e30
        for _ in range(5):
            e0, e1 = _events(torch)
            e0.record()
            bt.launch()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        print("batch_3d_small: %.3f ms, %.1f GCell-updates/s" % (best, cells / best / 1e6))
    elif case == "batch_one_launch_mix":
        # a scaled-down mix of the benchmark batch in the one-launch engine:
        # 48 2-D R=1 grids (sides 64..1024, about half ragged) and 16 3-D R=2
        # grids (sides 32..160), 40..200 sweeps; one kernel per launch, about
        # 0.3 GB on the device
        import numpy as np
        rng = np.random.default_rng(5)
        jobs, cells = [], 0
        for k in range(64):
            if k < 48:
                n, R = int(round(np.exp(rng.uniform(np.log(64), np.log(1024))))), 1
                shape = (n, n)
            else:
                n, R = int(round(np.exp(rng.uniform(np.log(32), np.log(160))))), 2
                shape = (n, n, n)
            it = int(rng.integers(40, 201))
            u = S.init_uniform(shape, k)
            jobs.append((u, u.clone(), R, it, J))
            c = it
            for d in shape:
                c *= d - 2 * R
            cells += c
        bt = S.Batch(jobs, engine="one_launch")
        for _ in range(3):
            bt.launch()
        best = 1e30
        for _ in range(5):
            e0, e1 = _events(torch)
            e0.record()
            bt.launch()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        print("batch_one_launch_mix: %.3f ms, %.1f GCell-updates/s, %d kernel per launch"
              % (best, cells / best / 1e6, bt.kernel_launches()))
    else:
        raise SystemExit("unknown profile case " + case)
    torch.cuda.synchronize()
    print("done", case)


def main():
    args = parse()
    if args.profile_case:
        _profile_case(args.profile_case)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
