"""Mixed-precision iterative refinement against the FP32 sweep loop and the
FP64 oracle (BF16 and FP16 correction storage, FP32 master, FP64 residual)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage,bound", [("bf16", 1e-3), ("fp16", 1.5e-4)])
# R = 4 runs the tensor-core correction sweep: partial tiles in x (nx = 136,
# 64) and y (ny = 72, 33), several z chunks (nz = 100)
@pytest.mark.parametrize("shape,radius,sweeps", [((64, 64, 64), 4, 200), ((40, 72, 136), 4, 120),
                                                 ((100, 33, 64), 4, 90), ((48, 56, 64), 2, 150),
                                                 ((256, 256), 1, 400)])
def test_ir_matches_fp32_and_fp64(cuda, storage, bound, shape, radius, sweeps):
    import torch
    from thesis_gb300 import stencil as S
    u0 = S.init_fourier(shape, 31, radius, modes=8)
    host = u0.cpu().numpy()
    # FP32 sweep loop
    a, b = u0.clone(), u0.clone()
    fp32 = S.sweep(a, b, radius, sweeps, O.JACOBI, "auto").cpu().numpy()
    # IR
    u = u0.clone()
    done, outer, rel = S.ir_solve(u, radius, sweeps, storage, inner_sweeps=50)
    got = u.cpu().numpy()
    assert done == sweeps and outer == -(-sweeps // 50)
    # FP64 oracle
    h64 = host.astype(np.float64)
    r64 = O.run(h64.copy(), h64.copy(), radius, O.JACOBI, sweeps, threads=8)
    # Fourier borders change sign, so errors are normwise: max |a - b| / max |b|
    # (an element-wise relative error is undefined at the zero crossings).
    scale = float(np.abs(r64).max())
    e32 = float(np.abs(fp32 - r64).max()) / scale
    eir = float(np.abs(got - r64).max()) / scale
    eir32 = float(np.abs(got - fp32).max()) / scale
    res32 = O.rel_residual(fp32, radius)
    print("%s %s R=%d: fp32-vs-fp64 %.3e  ir-vs-fp64 %.3e  ir-vs-fp32 %.3e  rel_res ir %.4e fp32 %.4e"
          % (storage, shape, radius, e32, eir, eir32, rel, res32))
    assert np.isfinite(got).all()
    assert e32 < 1e-6
    assert eir < bound and eir32 < bound
    assert rel == pytest.approx(res32, rel=0.05)  # equal accuracy at equal sweep counts
    # the border band is untouched
    band = np.ones(shape, bool)
    band[(slice(radius, -radius),) * len(shape)] = False
    assert np.array_equal(got[band], host[band])
    # residual as reported equals the oracle's (all-FP64) residual of the
    # returned grid, up to the FP32 per-cell evaluation
    assert rel == pytest.approx(O.rel_residual(got, radius), rel=1e-6)


def test_ir_converges_to_tolerance(cuda):
    from thesis_gb300 import stencil as S
    shape = (128, 128)
    u = S.init_laplace2d(shape, 9)
    done, outer, rel = S.ir_solve(u, 1, 200000, "fp16", inner_sweeps=100, tol=1e-4,
                                  check_every=5)
    assert rel < 1e-4 and done < 200000
    assert O.rel_residual(u.cpu().numpy(), 1) < 1e-4


def test_ir_rejects_legacy_and_bad_storage(cuda):
    import ctypes, torch
    from thesis_gb300 import lib as L
    u = torch.zeros((32, 32), device="cuda")
    p = L.make_params((32, 32), 1, 10, L.MODE_LEGACY)
    ir = L.IrParams()
    ir.storage = L.STORAGE_BF16
    res = L.IrResult()
    ws = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    assert L.load().stencil_ir_solve(ctypes.byref(p), ctypes.byref(ir), ctypes.c_void_p(u.data_ptr()),
                                     ctypes.c_void_p(ws.data_ptr()), ws.numel(), None,
                                     ctypes.byref(res)) == L.EINVAL
    p.mode = L.MODE_JACOBI
    ir.storage = L.STORAGE_FP32
    assert L.load().stencil_ir_solve(ctypes.byref(p), ctypes.byref(ir), ctypes.c_void_p(u.data_ptr()),
                                     ctypes.c_void_p(ws.data_ptr()), ws.numel(), None,
                                     ctypes.byref(res)) == L.EINVAL


def test_borders_generators(cuda):
    from thesis_gb300 import stencil as S
    a = S.init_fourier((20, 24, 28), 5, 2).cpu().numpy()
    b = S.init_fourier((20, 24, 28), 5, 2).cpu().numpy()
    assert np.array_equal(a, b) and np.isfinite(a).all()
    inner = a[2:-2, 2:-2, 2:-2]
    assert inner.min() >= 0 and inner.max() < 1
    lap = S.init_laplace2d((2048, 2048), 3).cpu().numpy()
    assert np.all(lap[1:-1, 1:-1] == 0)
    # continuous at the corners: on a fine grid the cells next to a corner
    # along both edges are close to the corner value
    for (j, i), (dj, di) in [((0, 0), (1, 1)), ((0, -1), (1, -1)), ((-1, 0), (-1, 1)), ((-1, -1), (-1, -1))]:
        c = lap[j, i]
        assert abs(lap[j, i + di] - c) < 0.5 and abs(lap[j + dj, i] - c) < 0.5
