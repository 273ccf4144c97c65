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
  3. solve: the predicted field seeds plain FP32 Jacobi, which runs to the
     relative residual tolerance; the prediction replaces zero only when its
     residual is lower (fallback rule).

The sweep counts to tolerance are found with all grids of an evaluation set in
one batched launch per chunk of sweeps and a residual check between chunks.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import lib as _lib
from . import stencil as S
from .unet import UNet


def coons_fill(fields):
    """Border kept, interior = transfinite interpolation of the border."""
    import torch
    f = fields
    n, h, w = f.shape
    s = torch.linspace(0, 1, w, device=f.device)[None, None, :]
    t = torch.linspace(0, 1, h, device=f.device)[None, :, None]
    B, T = f[:, :1, :], f[:, -1:, :]
    L, R = f[:, :, :1], f[:, :, -1:]
    c00, c10 = f[:, :1, :1], f[:, :1, -1:]
    c01, c11 = f[:, -1:, :1], f[:, -1:, -1:]
    cp = ((1 - t) * B + t * T + (1 - s) * L + s * R -
          ((1 - s) * (1 - t) * c00 + s * (1 - t) * c10 + (1 - s) * t * c01 + s * t * c11))
    out = cp.clone()
    out[:, 0, :], out[:, -1, :], out[:, :, 0], out[:, :, -1] = f[:, 0, :], f[:, -1, :], f[:, :, 0], f[:, :, -1]
    return out.contiguous()


def borders(seeds, size, device="cuda"):
    import torch
    return torch.stack([S.init_laplace2d((size, size), int(s), device=device) for s in seeds])


def run_batch(grids_a, grids_b, sweeps, cluster_size=0):
    """Runs `sweeps` Jacobi sweeps on each grid pair in one persistent launch;
    returns the tensors holding the results."""
    jobs = [(a, b, 1, int(sweeps), _lib.MODE_JACOBI) for a, b in zip(grids_a, grids_b)]
    bt = S.Batch(jobs, cluster_size=cluster_size)
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


def predict(net, fields, mode="direct", train_size=128):
    """Initial fields for `fields` (n, H, W).  mode 'direct' applies the fully
    convolutional network at H x W; 'coarse' applies it to the border sampled
    at train_size x train_size and interpolates the prediction bilinearly."""
    import torch
    if mode == "direct":
        return net.predict(fields)
    n, H, W = fields.shape
    idx_y = torch.round(torch.linspace(0, H - 1, train_size, device=fields.device)).long()
    idx_x = torch.round(torch.linspace(0, W - 1, train_size, device=fields.device)).long()
    coarse = fields[:, idx_y][:, :, idx_x].contiguous()
    # border of the coarse problem only (interior zero)
    cf = torch.zeros_like(coarse)
    cf[:, 0, :], cf[:, -1, :], cf[:, :, 0], cf[:, :, -1] = coarse[:, 0, :], coarse[:, -1, :], coarse[:, :, 0], coarse[:, :, -1]
    pc = net.predict(cf.contiguous())
    up = torch.nn.functional.interpolate(pc[:, None], size=(H, W), mode="bilinear",
                                         align_corners=True)[:, 0]
    out = up.clone()
    out[:, 0, :], out[:, -1, :], out[:, :, 0], out[:, :, -1] = fields[:, 0, :], fields[:, -1, :], fields[:, :, 0], fields[:, :, -1]
    return out.contiguous()


def residuals(grids):
    return [S.residual(g, 1) for g in grids]


def sweeps_to_tol(inits, tol=1e-5, chunk=2000, max_sweeps=400000):
    """Plain FP32 Jacobi from each initial field until the FP64 relative
    residual is below tol; all unconverged grids advance together in one
    batched launch per chunk.  Returns (sweeps per grid, device seconds)."""
    import torch
    n = len(inits)
    cur = [u.clone() for u in inits]
    other = [u.clone() for u in inits]
    done = [0] * n
    active = [k for k in range(n) if S.residual(cur[k], 1) >= tol]
    elapsed = 0.0
    while active:
        step = chunk
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        res = run_batch([cur[k] for k in active], [other[k] for k in active], step)
        e1.record()
        e1.synchronize()
        elapsed += e0.elapsed_time(e1) / 1e3
        nxt = []
        for k, r in zip(active, res):
            if r.data_ptr() != cur[k].data_ptr():
                cur[k], other[k] = r, cur[k]
            done[k] += step
            if S.residual(cur[k], 1) >= tol and done[k] < max_sweeps:
                nxt.append(k)
        active = nxt
    return done, elapsed


def per_sweep_seconds(size=512, sweeps=2000):
    """Time of one FP32 sweep of one size x size grid on the plain kernel
    (cluster engine, shared-memory resident)."""
    import torch
    u = S.init_laplace2d((size, size), 5)
    a, b = u.clone(), u.clone()
    S.sweep(a, b, 1, 200, _lib.MODE_JACOBI, "auto")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    S.sweep(a, b, 1, sweeps, _lib.MODE_JACOBI, "auto")
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / sweeps


def evaluate(net, seeds, size=512, tol=1e-5, chunk=2000, log=print):
    """Sweeps and time to tol for each arm on the held-out seeds."""
    import torch
    f = borders(seeds, size)
    arms = {}
    t_sweep = per_sweep_seconds(size)
    # plain: zero interior
    arms["zero"] = f.clone()
    arms["coons"] = coons_fill(f)
    torch.cuda.synchronize()
    t0 = time.time()
    for mode in ("direct", "coarse"):
        predict(net, f, mode)  # warm-up: allocates the activation buffers for this shape
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        p = predict(net, f, mode)
        e1.record()
        e1.synchronize()
        arms["net_" + mode] = p
        arms["net_" + mode + "_infer_s"] = e0.elapsed_time(e1) / 1e3 / len(seeds)
    out = {"per_sweep_s": t_sweep, "size": size, "tol": tol, "n": len(seeds)}
    r_zero = residuals(list(arms["zero"]))
    for name in ("zero", "coons", "net_direct", "net_coarse"):
        inits = list(arms[name])
        r0 = residuals(inits)
        # fallback rule: keep the prediction only where its residual is lower than zero init's
        chosen = [inits[k] if r0[k] < r_zero[k] else arms["zero"][k] for k in range(len(inits))]
        used = sum(1 for k in range(len(inits)) if r0[k] < r_zero[k])
        sw, dev_s = sweeps_to_tol(chosen, tol, chunk)
        infer = arms.get(name + "_infer_s", 0.0)
        out[name] = {"mean_sweeps": float(np.mean(sw)), "median_sweeps": float(np.median(sw)),
                     "initial_residual_median": float(np.median(r0)), "prediction_used": used,
                     "time_per_solve_s": float(np.mean(sw)) * t_sweep + infer,
                     "infer_s_per_grid": infer}
        log("%-11s sweeps mean %.0f  r0 median %.3e  used %d/%d  time/solve %.4f s"
            % (name, out[name]["mean_sweeps"], out[name]["initial_residual_median"], used,
               len(inits), out[name]["time_per_solve_s"]))
    for name in ("coons", "net_direct", "net_coarse"):
        out[name]["speedup_vs_zero"] = out["zero"]["time_per_solve_s"] / out[name]["time_per_solve_s"]
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
