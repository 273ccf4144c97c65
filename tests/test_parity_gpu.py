"""GPU parity: every kernel family against the CPU oracle, bit for bit.

All kernels keep the reference's per-cell summation order
(src/stencils.cu:8-19), so the bar is bit-exact equality of the whole result
buffer (border band included) with the oracle run on the same input.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "legacy_*.npz")))
VARIANTS = ["base", "smem", "smem_padded", "smem_register", "coop", "cluster", "auto"]


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def gpu_run(u_host, radius, iters, mode, variant, second=None, **kw):
    import torch
    from thesis_gb300 import stencil as S
    u1 = torch.from_numpy(u_host).cuda()
    u2 = torch.from_numpy(second if second is not None else u_host).cuda()
    res = S.sweep(u1, u2, radius, iters, mode, variant, **kw)
    torch.cuda.synchronize()
    return res.cpu().numpy(), u1, u2, res


def oracle_run(u_host, radius, iters, mode, second=None, threads=8):
    a = u_host.copy()
    b = (second if second is not None else u_host).copy()
    return O.run(a, b, radius, mode, iters, threads=threads)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("variant", ["base", "smem_padded", "smem_register", "coop", "auto"])
def test_golden_legacy(cuda, path, variant):
    """The reference's own stencil_cpu output, reproduced by each GPU variant."""
    import torch
    from thesis_gb300 import stencil as S
    z = np.load(path)
    grid, radius, iters = z["grid"], int(z["radius"]), int(z["iterations"])
    u1 = S.init_reference(grid.shape)
    u2 = torch.zeros_like(u1)
    res = S.sweep(u1, u2, radius, iters, O.LEGACY, variant)
    assert bits_equal(res.cpu().numpy(), grid)


CASES = [
    # (shape, radius, iterations)
    ((64, 64), 1, 10), ((67, 130), 2, 7), ((256, 256), 1, 25), ((100, 96), 4, 6),
    ((33, 48), 8, 3), ((80, 64), 16, 2),
    ((32, 32, 32), 1, 9), ((40, 36, 64), 2, 5), ((48, 48, 48), 4, 6), ((30, 31, 37), 3, 4),
    ((20, 24, 128), 1, 12), ((40, 40, 40), 8, 2), ((9, 9, 12), 4, 3),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[0])) + "_r%d_i%d" % c[1:])
@pytest.mark.parametrize("mode", [O.LEGACY, O.JACOBI], ids=["legacy", "jacobi"])
@pytest.mark.parametrize("variant", VARIANTS)
def test_variant_matches_oracle(cuda, case, mode, variant):
    shape, radius, iters = case
    u = O.uniform(shape, seed=hash((shape, radius, iters)) & 0xFFFF)
    second = None
    if mode == O.LEGACY:
        second = O.uniform(shape, seed=77)  # arbitrary second-buffer border
    got, *_ = gpu_run(u, radius, iters, mode, variant, second)
    want = oracle_run(u, radius, iters, mode, second)
    assert bits_equal(got, want)


@pytest.mark.parametrize("variant", ["base", "smem_padded", "smem_register"])
@pytest.mark.parametrize("iters", [0, 1, 2, 3])
def test_result_buffer_and_odd_counts(cuda, variant, iters):
    """The returned buffer is the one holding sweep `iters` (the reference reads
    back d_u1 even for odd counts, src/main.cu:79; this library reports it)."""
    u = O.uniform((24, 40, 64), seed=3)
    got, u1, u2, res = gpu_run(u, 1, iters, O.JACOBI, variant)
    assert (res.data_ptr() == u1.data_ptr()) == (iters % 2 == 0)
    assert bits_equal(got, oracle_run(u, 1, iters, O.JACOBI))


@pytest.mark.parametrize("block", [(8, 2, 2), (32, 4, 1), (16, 1, 8), (4, 16, 4)])
@pytest.mark.parametrize("variant", ["base", "smem"])
def test_block_shapes(cuda, block, variant):
    u = O.uniform((36, 50, 72), seed=9)
    got, *_ = gpu_run(u, 2, 3, O.JACOBI, variant, block=block, coarsen_x=8)
    assert bits_equal(got, oracle_run(u, 2, 3, O.JACOBI))


def test_device_init_matches_oracle_generators(cuda):
    from thesis_gb300 import stencil as S
    shape = (17, 33, 65)
    assert bits_equal(S.init_uniform(shape, 1234).cpu().numpy(), O.uniform(shape, 1234))
    assert bits_equal(S.init_reference(shape).cpu().numpy(), O.init_reference(shape))
    assert bits_equal(S.init_reference((31, 45)).cpu().numpy(), O.init_reference((31, 45)))


def test_copy_border(cuda):
    import torch
    from thesis_gb300 import stencil as S
    src = S.init_uniform((20, 21, 22), 5)
    dst = torch.full_like(src, -3.0)
    S.copy_border(src, dst, 3)
    want = np.full((20, 21, 22), -3.0, np.float32)
    O.copy_border(src.cpu().numpy(), want, 3)
    assert bits_equal(dst.cpu().numpy(), want)


@pytest.mark.parametrize("shape,radius", [((96, 80), 1), ((30, 40, 50), 2), ((64, 64), 3)])
def test_residual_matches_oracle(cuda, shape, radius):
    from thesis_gb300 import stencil as S
    u = S.init_uniform(shape, 21)
    got = S.residual(u, radius)
    want = O.rel_residual(u.cpu().numpy(), radius)
    # per-cell residual in FP32 (neighbour - centre differences), squares in FP64
    assert got == pytest.approx(want, rel=1e-6)


def test_run_host_matches_dispatch(cuda):
    from thesis_gb300 import stencil as S
    u = O.uniform((48, 40, 64), seed=8)
    out, ms = S.run_host(u, 2, 7, O.JACOBI)
    assert ms > 0
    assert bits_equal(out, oracle_run(u, 2, 7, O.JACOBI))
    out_l, _ = S.run_host(u, 2, 7, O.LEGACY)
    assert bits_equal(out_l, oracle_run(u, 2, 7, O.LEGACY, np.zeros_like(u)))


def test_run_host_pinned_buffers_match_pageable(cuda, monkeypatch):
    """Pinned (mapped) host buffers are copied by the streaming kernel, pageable
    ones and unaligned views by the copy engines: the same bits either way."""
    import torch
    from thesis_gb300 import stencil as S
    u = O.uniform((64, 72, 80), seed=9)
    want = oracle_run(u, 1, 5, O.JACOBI)
    pin_in = torch.from_numpy(u.copy()).pin_memory()
    pin_out = torch.zeros_like(pin_in).pin_memory()
    out, _ = S.run_host(pin_in.numpy(), 1, 5, O.JACOBI, out=pin_out.numpy())
    assert out.ctypes.data == pin_out.data_ptr()
    assert bits_equal(pin_out.numpy(), want)
    pageable, _ = S.run_host(u, 1, 5, O.JACOBI)
    assert bits_equal(pageable, want)
    monkeypatch.setenv("STENCIL_HOST_COPY", "engine")
    pin_out.zero_()
    S.run_host(pin_in.numpy(), 1, 5, O.JACOBI, out=pin_out.numpy())
    assert bits_equal(pin_out.numpy(), want)
    # a pinned view one float in: not 16-byte aligned, so the copy engines
    monkeypatch.delenv("STENCIL_HOST_COPY")
    flat_in = torch.from_numpy(np.concatenate([[0.0], u.ravel()]).astype(np.float32)).pin_memory()
    flat_out = torch.zeros_like(flat_in).pin_memory()
    S.run_host(flat_in.numpy()[1:].reshape(u.shape), 1, 5, O.JACOBI,
               out=flat_out.numpy()[1:].reshape(u.shape))
    assert bits_equal(flat_out.numpy()[1:].reshape(u.shape), want)


def test_no_device_faults_reported(cuda):
    from thesis_gb300 import stencil as S
    assert S.device_status() == 0


@pytest.mark.slow
@pytest.mark.parametrize("radius", [1, 4])
def test_full_size_512_cubed(cuda, radius):
    """512^3 (the benchmark grid): 3 sweeps against the oracle (all host cores),
    and the variants against each other for 20 sweeps."""
    import torch
    from thesis_gb300 import stencil as S
    shape = (512, 512, 512)
    u = S.init_uniform(shape, 2024)
    host = u.cpu().numpy()
    want = oracle_run(host, radius, 3, O.JACOBI, threads=os.cpu_count() or 8)
    outs = {}
    for variant in ["base", "smem_register", "auto"]:
        a, b = u.clone(), u.clone()
        res = S.sweep(a, b, radius, 3, O.JACOBI, variant)
        assert bits_equal(res.cpu().numpy(), want), variant
        a, b = u.clone(), u.clone()
        outs[variant] = S.sweep(a, b, radius, 20, O.JACOBI, variant).cpu().numpy()
        del a, b
        torch.cuda.empty_cache()
    assert bits_equal(outs["base"], outs["smem_register"])
    assert bits_equal(outs["base"], outs["auto"])


TB_CASES = [((64, 64, 64), 1, 2, 8), ((64, 64, 64), 1, 3, 9), ((64, 64, 64), 1, 4, 13),
            ((40, 52, 100), 1, 4, 11), ((30, 36, 48), 2, 2, 7), ((12, 12, 12), 1, 4, 8),
            ((9, 20, 136), 1, 4, 4), ((100, 70, 260), 2, 2, 4)]


@pytest.mark.parametrize("case", TB_CASES, ids=lambda c: "x".join(map(str, c[0])) + "_r%d_T%d_i%d" % c[1:])
def test_temporal_blocking_matches_oracle(cuda, case):
    """COOP: T sweeps per HBM pass with overlapped tiles, bit-exact with the oracle."""
    shape, radius, T, iters = case
    u = O.uniform(shape, seed=17)
    got, *_ = gpu_run(u, radius, iters, O.JACOBI, "coop", temporal=T)
    assert bits_equal(got, oracle_run(u, radius, iters, O.JACOBI))


@pytest.mark.slow
def test_temporal_blocking_full_size(cuda):
    """512^3: the temporally blocked passes equal the single-sweep kernel bit for bit."""
    import torch
    from thesis_gb300 import stencil as S
    u = S.init_uniform((512, 512, 512), 99)
    outs = []
    for variant, T in (("smem_register", 0), ("coop", 4), ("coop", 3)):
        a, b = u.clone(), u.clone()
        outs.append(S.sweep(a, b, 1, 24, O.JACOBI, variant, temporal=T).cpu().numpy())
        del a, b
        torch.cuda.empty_cache()
    assert bits_equal(outs[0], outs[1]) and bits_equal(outs[0], outs[2])


def special_values_grid(shape, seed):
    """Uniform field with regions of -0.0, +0.0, subnormals, huge values
    (sums overflow to inf), NaN and alternating signs, so every division path
    and every signed-zero case of the sum meets the oracle."""
    rng = np.random.default_rng(seed)
    u = O.uniform(shape, seed=seed)
    flat = u.reshape(-1)
    n = flat.size
    picks = rng.integers(0, 8, n)
    flat[picks == 1] = -0.0
    flat[picks == 2] = 0.0
    flat[picks == 3] = np.float32(1e-39) * rng.choice([-1, 1], (picks == 3).sum())
    flat[picks == 4] = np.float32(3e38) * rng.choice([-1, 1], (picks == 4).sum())
    flat[picks == 5] = -flat[picks == 5]
    flat[rng.integers(0, n, 3)] = np.nan
    # a block of all -0.0 so that whole neighbourhoods sum -0 terms only
    sl = tuple(slice(2, 2 + 12) for _ in shape)
    u[sl] = -0.0
    return u


@pytest.mark.parametrize("shape,radius", [((40, 40, 64), 1), ((40, 40, 64), 2), ((36, 40, 72), 3),
                                          ((36, 40, 72), 4), ((64, 96), 1), ((64, 96), 3)])
@pytest.mark.parametrize("variant", ["base", "smem_padded", "smem_register", "coop", "cluster"])
@pytest.mark.parametrize("mode", [O.LEGACY, O.JACOBI], ids=["legacy", "jacobi"])
def test_special_values_match_oracle(cuda, shape, radius, variant, mode):
    u = special_values_grid(shape, radius * 7 + len(shape))
    got, *_ = gpu_run(u, radius, 2, mode, variant, u.copy())
    want = oracle_run(u, radius, 2, mode, u.copy())
    # NaN payloads differ between CPUs and GPUs (the GPU returns its canonical
    # NaN); NaN positions and every other bit pattern must agree.
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_g, nan_w)
    assert np.array_equal(got[~nan_g].view(np.uint32), want[~nan_w].view(np.uint32))


PERSISTENT_CASES = [((40, 36, 64), 1, 0), ((40, 36, 64), 1, 1), ((40, 36, 64), 1, 7),
                    ((48, 40, 72), 2, 6), ((36, 44, 136), 3, 5), ((48, 48, 48), 4, 4),
                    ((20, 24, 260), 1, 9), ((72, 130, 260), 2, 3)]


@pytest.mark.parametrize("case", PERSISTENT_CASES, ids=lambda c: "x".join(map(str, c[0])) + "_r%d_i%d" % c[1:])
@pytest.mark.parametrize("mode", [O.LEGACY, O.JACOBI], ids=["legacy", "jacobi"])
def test_persistent_stream_matches_oracle(cuda, case, mode):
    """COOP with temporal = 1: every sweep in one cooperative launch, a
    grid-wide barrier between sweeps; bit-exact, result buffer by parity."""
    shape, radius, iters = case
    u = O.uniform(shape, seed=31 + radius)
    second = O.uniform(shape, seed=32) if mode == O.LEGACY else None
    got, u1, u2, res = gpu_run(u, radius, iters, mode, "coop", second, temporal=1)
    assert (res.data_ptr() == u1.data_ptr()) == (iters % 2 == 0)
    assert bits_equal(got, oracle_run(u, radius, iters, mode, second))


@pytest.mark.slow
@pytest.mark.parametrize("variant", ["auto", "base"])
def test_grid_beyond_2_31_cells(cuda, variant):
    """1296^3 = 2.18e9 cells (8.7 GB per buffer): 2 sweeps, then planes near
    the middle and the far end (offsets beyond 2^31 cells) against the oracle
    run on the 5-plane slab that determines them."""
    import torch
    from thesis_gb300 import stencil as S
    n, R, iters = 1296, 1, 2
    u = S.init_uniform((n, n, n), 77)
    a, b = u.clone(), u.clone()
    res = S.sweep(a, b, R, iters, O.JACOBI, variant)
    torch.cuda.synchronize()
    for z in (n // 2, n - 3):
        slab = u[z - 2:z + 3].cpu().numpy()
        want = oracle_run(slab, R, iters, O.JACOBI, threads=os.cpu_count() or 8)
        got = res[z].cpu().numpy()
        assert bits_equal(got, want[2]), z
    del a, b, u, res
    torch.cuda.empty_cache()
