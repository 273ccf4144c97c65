"""Learned warm start for 2-D Laplace steady-state solves.

Pipeline:
  1. data: Dirichlet borders from stencil_init_laplace2d (per edge K~U{1..16}
     sine modes with N(0,1) amplitudes plus the linear interpolation of four
     N(0,1) corner values); the solutions come from this library's own Jacobi
     solver -- one batched persistent launch (stencil_batch_*, one CTA per
     128x128 grid resident in shared memory) from the transfinite (Coons)
     interpolation of the border;
  2. training: the U-Net of unet.py, every kernel hand-written (BF16 tensor
     cores, FP32 accumulation), Adam on FP32 master weights;
  3. solve: the network, applied to the border resampled to the training size,
     predicts the initial field (bilinear back to the grid); the solver runs
     from it to the relative residual tolerance -- plain FP32 Jacobi, or the
     mixed-precision refinement (FP16/BF16 correction sweeps, FP32 master,
     FP64 residual norm; stencil_ir_solve) -- and the prediction replaces zero
     only when its residual is lower (fallback rule).

Every solve is timed with CUDA events around all of its GPU work: the
network's inference, the fallback check, every sweep and every residual
check (one every 500 sweeps for the plain loop; one per outer step of the
refinement).  The plain loop this accelerates is the reference's sweep loop
(src/stencil_cpu.cu:32-35, src/stencil_dispatch.cu:153-157).
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import lib as _lib
from . import stencil as S
from . import unet as U
from .unet import UNet

CHECK_EVERY = 500        # sweeps between residual checks of the plain loop
TRAIN_SIZE = 128         # grid side the network is trained (and applied) at
IR_INNER = {"fp16": 500, "bf16": 100}  # correction sweeps per outer step


def coons_fill(fields):
    """Border kept, interior = transfinite interpolation of the border."""
    return U.coons_fill(fields.contiguous())


def borders(seeds, size, device="cuda"):
    import torch
    return torch.stack([S.init_laplace2d((size, size), int(s), device=device) for s in seeds])


def run_batch(grids_a, grids_b, sweeps, cluster_size=0):
    """Runs `sweeps` Jacobi sweeps on each grid pair in one persistent launch;
    returns the tensors holding the results."""
    jobs = [(a, b, 1, int(sweeps), _lib.MODE_JACOBI) for a, b in zip(grids_a, grids_b)]
    bt = S.Batch(jobs, cluster_size=cluster_size, engine="phased")
    bt.launch()
    res = [bt.result(k) for k in range(len(jobs))]
    bt.close()
    return res


def generate_pairs(n, size=128, seed0=1_000_000, sweeps=40000, chunk=4096):
    """n (border field, Jacobi solution) pairs at size x size."""
    import torch
    fields = torch.empty((n, size, size), device="cuda")
    sols = torch.empty((n, size, size), device="cuda")
    for k0 in range(0, n, chunk):
        k1 = min(n, k0 + chunk)
        f = borders(range(seed0 + k0, seed0 + k1), size)
        a = coons_fill(f)
        b = a.clone()
        res = run_batch(list(a), list(b), sweeps, cluster_size=1)
        fields[k0:k1] = f
        sols[k0:k1] = torch.stack(res)
    torch.cuda.synchronize()
    return fields, sols


def train(net, fields, sols, epochs=8, batch=64, lr=2e-3, log=None):
    import torch
    n = fields.shape[0]
    g = torch.Generator(device="cpu").manual_seed(1)
    steps = 0
    losses = []
    total_steps = epochs * (n // batch)
    t0 = time.time()
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).cuda()
        ep_loss = 0.0
        for k in range(n // batch):
            idx = perm[k * batch:(k + 1) * batch]
            f = fields[idx].contiguous()
            y = sols[idx].contiguous()
            net.zero_grad()
            B = net.loss_and_grad(f, y)
            net.backward(B)
            # cosine learning-rate decay
            cur = lr * 0.5 * (1 + math.cos(math.pi * steps / max(1, total_steps)))
            net.adam_step(lr=cur)
            steps += 1
            if k % 50 == 0:
                ep_loss = B["loss"].item() / (batch * (f.shape[1] - 2) * (f.shape[2] - 2))
                losses.append(ep_loss)
        if log:
            log("epoch %d loss %.3e (%.1f s)" % (ep, ep_loss, time.time() - t0))
    torch.cuda.synchronize()
    return losses, time.time() - t0


def predict(net, fields, mode="coarse", train_size=TRAIN_SIZE):
    """Initial fields for `fields` (n, H, W).  mode 'direct' applies the fully
    convolutional network at H x W; 'coarse' applies it to the border sampled
    at train_size x train_size and interpolates the prediction bilinearly
    (every step a kernel of this library)."""
    if mode == "direct":
        return net.predict(fields)
    coarse = U.resample_border(fields, train_size, train_size)
    pc = net.predict(coarse)
    return U.upsample_bilinear(pc, fields)


def residuals(grids):
    return [S.residual(g, 1) for g in grids]


def solve_plain(u_init, tol=1e-5, check=CHECK_EVERY, max_sweeps=2_000_000):
    """Plain FP32 Jacobi (the library's AUTO engine, bit-exact sweeps) from
    u_init until the relative residual is below tol, checked every `check`
    sweeps (stencil_solve: the loop runs in the library).  Returns (sweeps,
    residual, result grid)."""
    a, b = u_init.clone(), u_init.clone()
    done, r, res = S.solve(a, b, 1, max_sweeps, tol, check)
    return done, r, res


def solve_ir(u_init, storage, tol=1e-5, inner=None, workspace=None, max_sweeps=2_000_000):
    """Mixed-precision refinement from u_init to tol (residual checked after
    every outer step).  Returns (sweeps, residual, result grid)."""
    u = u_init.clone()
    r = S.ir_solve_ex(u, 1, max_sweeps, storage, inner_sweeps=inner or IR_INNER[storage], tol=tol,
                      check_every=1, workspace=workspace)
    return r["sweeps"], r["rel_residual"], u


def timed(fn):
    """(fn's result, seconds) with CUDA events on the current stream around it."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    out = fn()
    e1.record()
    e1.synchronize()
    return out, e0.elapsed_time(e1) / 1e3


def warm_init(net, field, mode="coarse", train_size=TRAIN_SIZE):
    """The learned initial field of one problem (1, H, W) with the fallback
    rule: the prediction only where its relative residual is below that of
    the zero interior, which is 1 (its residual is the border term b itself)."""
    pred = predict(net, field, mode, train_size)[0]
    used = S.residual(pred, 1) < 1.0
    return (pred if used else field[0]), used


ARMS = {
    # name: (initial field, solver)
    "zero_fp32": ("zero", "fp32"),
    "zero_ir_fp16": ("zero", "fp16"),
    "learned_fp32": ("learned", "fp32"),
    "learned_ir_fp16": ("learned", "fp16"),
    "learned_ir_bf16": ("learned", "bf16"),
    "coons_fp32": ("coons", "fp32"),
    "direct_fp32": ("direct", "fp32"),
}


def solve_arm(net, field, arm, tol, ws, train_size=TRAIN_SIZE, check=CHECK_EVERY):
    """One timed solve of problem `field` (1, H, W): returns (sweeps,
    residual, seconds, prediction used, result).  `check`: sweeps between
    the plain loop's residual checks."""
    init, solver = ARMS[arm]

    def run():
        used = False
        if init == "zero":
            u0 = field[0]
        elif init == "coons":
            u0, used = coons_fill(field)[0], True
        else:
            u0, used = warm_init(net, field, "coarse" if init == "learned" else "direct",
                                 train_size)
        if solver == "fp32":
            sw, r, u = solve_plain(u0, tol, check)
        else:
            sw, r, u = solve_ir(u0, solver, tol, workspace=ws[solver])
        return sw, r, used, u

    (sw, r, used, u), sec = timed(run)
    return sw, r, sec, used, u


def exact_steady_state(field):
    """The FP64 steady state of one problem (H, W numpy array, border on the
    outer ring), the accuracy check of the solves (not part of them): the
    5-point Laplace system (4 u - sum of the 4 neighbours = border terms) is
    diagonalised by the type-I discrete sine transform in each axis, with
    eigenvalues 4 - 2 cos(p pi/(w+1)) - 2 cos(q pi/(h+1)), so one forward
    transform, a division and one inverse transform solve it to FP64
    rounding."""
    from scipy import fft
    f = np.asarray(field, np.float64)
    H, W = f.shape
    h, w = H - 2, W - 2
    b = np.zeros((h, w))
    b[0, :] += f[0, 1:-1]
    b[-1, :] += f[-1, 1:-1]
    b[:, 0] += f[1:-1, 0]
    b[:, -1] += f[1:-1, -1]
    lam = (4.0 - 2.0 * np.cos(np.pi * np.arange(1, h + 1) / (h + 1))[:, None]
           - 2.0 * np.cos(np.pi * np.arange(1, w + 1) / (w + 1))[None, :])
    out = f.copy()
    out[1:-1, 1:-1] = fft.idstn(fft.dstn(b, type=1) / lam, type=1)
    return out


def evaluate(net, seeds, size=512, tol=1e-5, arms=None, n_exact=4, log=print):
    """Iterations, time and accuracy to tol of every arm on the held-out
    seeds, one problem at a time on the whole GPU."""
    import torch
    arms = list(arms or ["zero_fp32", "learned_fp32", "learned_ir_fp16", "learned_ir_bf16",
                         "zero_ir_fp16"])
    fields = borders(seeds, size)
    ws = {st: S.ir_workspace((size, size), 1, st) for st in ("fp16", "bf16")}
    # warm-up: kernels loaded, network buffers and engine plans made (untimed)
    for arm in arms:
        solve_arm(net, fields[:1], arm, 1e-2, ws)
    torch.cuda.synchronize()
    exact = {}
    for k in range(min(n_exact, len(seeds))):
        try:
            exact[k] = exact_steady_state(fields[k].cpu().numpy())
        except ImportError:
            break
    out = {"size": size, "tol": tol, "n": len(seeds), "check_every_plain": CHECK_EVERY,
           "ir_inner_sweeps": dict(IR_INNER), "timing": "CUDA events around each solve "
           "(inference, fallback check, sweeps, residual checks); one problem at a time"}
    for arm in arms:
        sweeps, secs, res, used, errs = [], [], [], 0, []
        for k in range(len(seeds)):
            sw, r, sec, u_used, u = solve_arm(net, fields[k:k + 1], arm, tol, ws)
            sweeps.append(sw)
            secs.append(sec)
            res.append(r)
            used += int(u_used)
            if k in exact:
                ex = exact[k]
                errs.append(float(np.abs(u.cpu().numpy().astype(np.float64) - ex).max() /
                                  np.abs(ex).max()))
        out[arm] = {"mean_sweeps": float(np.mean(sweeps)), "median_sweeps": float(np.median(sweeps)),
                    "time_per_solve_s": float(np.mean(secs)),
                    "median_time_s": float(np.median(secs)),
                    "max_rel_residual": float(np.max(res)), "prediction_used": used,
                    "fp64_normwise_err_max": max(errs) if errs else None,
                    "fp64_err_seeds": len(errs)}
        log("%-16s sweeps mean %8.0f  time/solve %.4f s  max residual %.2e  used %d/%d  "
            "err vs FP64 %s" % (arm, out[arm]["mean_sweeps"], out[arm]["time_per_solve_s"],
                                out[arm]["max_rel_residual"], used, len(seeds),
                                "%.2e" % max(errs) if errs else "-"))
    base = out.get("zero_fp32")
    if base:
        for arm in arms:
            if arm != "zero_fp32":
                out[arm]["speedup_vs_plain"] = base["time_per_solve_s"] / out[arm]["time_per_solve_s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--gen-sweeps", type=int, default=40000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--eval", type=int, default=256)
    ap.add_argument("--eval-size", type=int, default=512)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--save", default=None)
    ap.add_argument("--json", default=None)
    args = ap.parse_args()
    import torch
    from . import build
    build.build()
    t0 = time.time()
    fields, sols = generate_pairs(args.pairs, args.size, sweeps=args.gen_sweeps)
    gen_s = time.time() - t0
    rres = [S.residual(sols[k], 1) for k in range(0, args.pairs, max(1, args.pairs // 16))]
    print("generated %d pairs in %.1f s, sample residual max %.2e" % (args.pairs, gen_s, max(rres)))
    net = UNet(seed=0)
    losses, train_s = train(net, fields, sols, args.epochs, args.batch, lr=args.lr, log=print)
    print("trained in %.1f s" % train_s)
    if args.save:
        net.save(args.save)
    del fields, sols
    torch.cuda.empty_cache()
    seeds = list(range(10_000_000, 10_000_000 + args.eval))
    res = evaluate(net, seeds, args.eval_size, args.tol)
    res.update({"pairs": args.pairs, "gen_s": gen_s, "train_s": train_s, "epochs": args.epochs,
                "lr": args.lr,
                "final_loss": losses[-1] if losses else None})
    print(json.dumps(res))
    if args.json:
        with open(args.json, "w") as fh:
            json.dump(res, fh, indent=1)


if __name__ == "__main__":
    main()
