"""The reference's own GPU kernels, compiled for sm_103a from their sources
(oracle/ref_gpu_kernels.cu) and launched with the reference's dispatch
geometry (oracle/ref_gpu.py): they reproduce the golden fixtures (so the
oracle, the reference kernels and this library agree bit for bit), and this
library sweeps faster than the best of them on the same GB300.

The cubins are built where the reference sources are (oracle/build.py,
build_ref_gpu); without them these tests skip."""
import os

import numpy as np
import pytest

from oracle import build as OB
from oracle import oracle as O
from oracle import ref_gpu as G

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


GOLDEN_CFGS = [((3, 64, 1, 32, 4, 4, 1), "legacy_3d_64_r1_i8.npz"),
               ((3, 64, 2, 32, 4, 4, 1), "legacy_3d_64_r2_i8.npz"),
               ((3, 64, 2, 32, 4, 4, 2), "legacy_3d_64_r2_i8.npz"),
               ((2, 64, 1, 32, 8, 1, 1), "legacy_2d_64_r1_i8.npz")]


@pytest.mark.parametrize("cfg,golden", GOLDEN_CFGS, ids=lambda x: str(x))
@pytest.mark.parametrize("variant", G.VARIANTS)
def test_reference_kernels_reproduce_golden(cuda, cfg, golden, variant):
    import torch
    if not G.available(cfg):
        pytest.skip("reference cubins not built (no reference sources where the package was built)")
    dims, dim, radius, bx, by, bz, cf = cfg
    want = np.load(os.path.join(os.path.dirname(__file__), "golden", golden))["grid"]
    u1 = torch.from_numpy(O.init_reference((dim,) * dims)).cuda()
    u2 = torch.zeros_like(u1)
    k = G.RefKernels(cfg)
    res = k.sweeps(variant, u1.data_ptr(), u2.data_ptr(), 8,
                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    k.close()
    out = (u1 if res == u1.data_ptr() else u2).cpu().numpy()
    assert bits_equal(out, want)


@pytest.mark.parametrize("radius", [1, 4])
def test_library_beats_reference_kernels_512(cuda, radius):
    """512^3 LEGACY: every reference kernel x block shape built for this
    radius runs on the same grid; the library matches each bit for bit after
    two sweeps and sweeps faster than the fastest of them."""
    import torch
    from thesis_gb300 import lib, stencil as S
    cfgs = [c for c in OB.REF_GPU_CONFIGS if c[1] == 512 and c[2] == radius]
    if not all(G.available(c) for c in cfgs):
        pytest.skip("reference cubins not built")
    n = 512
    u = S.init_uniform((n, n, n), 4242)
    a, b = u.clone(), torch.zeros_like(u)
    stream = torch.cuda.current_stream().cuda_stream
    sweeps, warm = 20, 3

    def timed(run):
        run(warm)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run(sweeps)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        return (n - 2 * radius) ** 3 * sweeps / best / 1e9

    # this library in LEGACY mode (the update the reference kernels compute), AUTO
    ours = timed(lambda k: S.sweep(a, b, radius, k, lib.MODE_LEGACY, "auto"))
    a.copy_(u)
    b.zero_()
    want = S.sweep(a, b, radius, 2, lib.MODE_LEGACY, "auto").clone()
    rows = []
    for cfg in cfgs:
        kern = G.RefKernels(cfg)
        for variant in G.VARIANTS:
            if not G.valid(variant, cfg[0], cfg[2], cfg[3], cfg[4], cfg[5]):
                continue
            a.copy_(u)
            b.zero_()
            res = kern.sweeps(variant, a.data_ptr(), b.data_ptr(), 2, stream)
            torch.cuda.synchronize()
            got = a if res == a.data_ptr() else b
            assert torch.equal(got.view(torch.int32), want.view(torch.int32)), (variant, cfg)
            v = timed(lambda k: kern.sweeps(variant, a.data_ptr(), b.data_ptr(), k, stream))
            rows.append((v, variant, tuple(cfg[3:])))
        kern.close()
    rows.sort(reverse=True)
    print("\n512^3 R=%d LEGACY: library %.1f GCell/s" % (radius, ours))
    for v, variant, shape in rows:
        print("  reference %-14s block %dx%dx%d cf %d: %.1f GCell/s" % ((variant,) + shape + (v,)))
    assert ours > rows[0][0]


def test_library_beats_reference_kernels_2d_256(cuda):
    """2-D 256^2 R=1, 1000 sweeps (the reference's 2-D configuration), LEGACY
    from the reference's initial state: every reference kernel x block shape
    built for it against the library's AUTO engine (one cooperative launch of
    the temporally blocked 2-D kernel), bit for bit and in time."""
    import torch
    from thesis_gb300 import lib, stencil as S
    cfgs = [c for c in OB.REF_GPU_CONFIGS if c[0] == 2 and c[1] == 256]
    if not all(G.available(c) for c in cfgs):
        pytest.skip("reference cubins not built")
    n, radius, sweeps = 256, 1, 1000
    u = torch.from_numpy(O.init_reference((n, n))).cuda()
    a, b = u.clone(), torch.zeros_like(u)
    def timed(run):
        run()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    def ours():
        a.copy_(u)
        b.zero_()
        return S.sweep(a, b, radius, sweeps, lib.MODE_LEGACY, "auto")

    ms_ours = timed(ours)
    want = ours().clone()
    rows = []
    for cfg in cfgs:
        kern = G.RefKernels(cfg)
        for variant in G.VARIANTS:
            if not G.valid(variant, cfg[0], cfg[2], cfg[3], cfg[4], cfg[5]):
                continue

            # the 1000 launches replayed from a CUDA graph: the reference
            # kernels without any host launch overhead
            graph, gs = torch.cuda.CUDAGraph(), torch.cuda.Stream()
            a.copy_(u)
            b.zero_()
            torch.cuda.synchronize()
            with torch.cuda.stream(gs):
                with torch.cuda.graph(graph, stream=gs):
                    res = kern.sweeps(variant, a.data_ptr(), b.data_ptr(), sweeps, gs.cuda_stream)

            def ref():
                a.copy_(u)
                b.zero_()
                graph.replay()

            ref()
            torch.cuda.synchronize()
            got = a if res == a.data_ptr() else b
            assert torch.equal(got.view(torch.int32), want.view(torch.int32)), (variant, cfg)
            rows.append((timed(ref), variant, tuple(cfg[3:])))
            del graph
        kern.close()
    rows.sort()
    print("\n256^2 R=1 LEGACY, 1000 sweeps: library %.3f ms (reference kernels replayed from CUDA graphs)" % ms_ours)
    for ms, variant, shape in rows:
        print("  reference %-14s block %dx%dx%d cf %d: %.3f ms" % ((variant,) + shape + (ms,)))
    assert ms_ours < rows[0][0]
