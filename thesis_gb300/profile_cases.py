"""Small, self-contained runs of each hot kernel, for profilers.

  python -m thesis_gb300.profile_cases <case>

Each case warms up, then runs the kernel a few more times; sizes are chosen so
that the working set exceeds the 129 MB L2 where the kernel is HBM-bound, yet a
full ncu capture of one launch ends in seconds.
"""
import sys
import time


def main(case):
    import torch
    from . import build, lib, stencil as S
    build.build()
    J = lib.MODE_JACOBI
    if case in ("stream_r1", "stream_r4", "stream_r1_512", "stream_r4_512"):
        R = 1 if case.startswith("stream_r1") else 4
        n = 512 if case.endswith("_512") else 320
        u = S.init_uniform((n, n, n), 1)  # 131 MB (320^3) or 537 MB (512^3) per buffer
        a, b = u.clone(), u.clone()
        for _ in range(4):
            S.sweep(a, b, R, 2, J, "smem_register")
    elif case in ("persist_r1_512", "persist_r4_512"):
        # the persistent engine AUTO runs: 8 sweeps in one cooperative launch
        R = 1 if case == "persist_r1_512" else 4
        u = S.init_uniform((512, 512, 512), 1)
        a, b = u.clone(), u.clone()
        for _ in range(3):
            S.sweep(a, b, R, 8, J, "coop", temporal=1)
    elif case in ("tb_r1_t2", "tb_r1_t4"):
        T = 2 if case.endswith("t2") else 4
        u = S.init_uniform((320, 320, 320), 1)
        a, b = u.clone(), u.clone()
        for _ in range(4):
            S.sweep(a, b, 1, T, J, "coop", temporal=T)
    elif case == "base_r1":
        u = S.init_uniform((320, 320, 320), 1)
        a, b = u.clone(), u.clone()
        for _ in range(4):
            S.sweep(a, b, 1, 2, J, "base")
    elif case == "cluster_2d256":
        u = S.init_uniform((256, 256), 1)
        a, b = u.clone(), u.clone()
        for _ in range(4):
            S.sweep(a, b, 1, 1000, J, "cluster")
    elif case == "tb2d_256":
        # the 2-D temporally blocked engine AUTO runs on 256^2, 1000 sweeps
        # per launch
        u = S.init_uniform((256, 256), 1)
        a, b = u.clone(), u.clone()
        for _ in range(4):
            S.sweep(a, b, 1, 1000, J, "auto")
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
        import ctypes
        from . import unet as U
        L = U._L()
        x = torch.randn(64, 32, 32, 384, device="cuda").to(torch.bfloat16)
        w = (torch.randn(128, 9, 384, device="cuda") * 0.05).to(torch.bfloat16)
        b = torch.zeros(128, device="cuda")
        y = torch.empty(64, 32, 32, 128, dtype=torch.bfloat16, device="cuda")
        eng = 1 if case == "conv_tc" else 2
        for _ in range(4):
            U._chk(L.unet_conv3x3_fwd_engine(ctypes.byref(U.view(x)), U._p(w), U._p(b),
                                             ctypes.byref(U.view(y)), 1, 1, eng, None), case)
    elif case == "unet_train":
        from .unet import UNet
        from . import warmstart as W
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
        bt = S.Batch(jobs)
        for _ in range(3):
            bt.launch()
    elif case == "batch_3d_small":
        # the cluster phase of the benchmark batch's small 3-D part: 18 grids
        # of 56^3 .. 104^3, R = 2, 100 sweeps each, swept from L2 by clusters
        jobs = []
        for k in range(18):
            n = 56 + 8 * (k % 7)
            u = S.init_uniform((n, n, n), k)
            jobs.append((u, u.clone(), 2, 100, J))
        bt = S.Batch(jobs)
        for _ in range(3):
            bt.launch()
        # event-timed rate of the batch (best of 5 launches)
        cells = sum((n - 4) ** 3 * 100 for n in (56 + 8 * (k % 7) for k in range(18)))
        best = 1e30
        for _ in range(5):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            bt.launch()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        print("batch_3d_small: %.3f ms, %.1f GCell-updates/s" % (best, cells / best / 1e6))
    else:
        raise SystemExit("unknown case " + case)
    torch.cuda.synchronize()
    print("done", case)


if __name__ == "__main__":
    main(sys.argv[1])
