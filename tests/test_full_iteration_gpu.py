"""The benchmark workload at its full iteration count: 512^3 FP32, R = 1,
1000 Jacobi sweeps from the benchmark's input (uniform [0,1) border and
interior, seed 20251203), on the engine the benchmark runs (AUTO: the
persistent stream kernel), bit for bit against the FP32 oracle -- the
restatement of the reference's stencil_cpu loop (src/stencil_cpu.cu:20-43),
OpenMP over the host cores without changing any cell's arithmetic.  The
oracle takes about 45 s on 16 cores.  The 2-D 256^2 workload is also checked
at 1000 sweeps, with its FP64 error."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SEED = 20251203
THREADS = len(os.sched_getaffinity(0)) or 8


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("shape", [(512, 512, 512), (256, 256)])
def test_benchmark_workload_full_iterations_bit_exact(cuda, shape):
    import torch
    from thesis_gb300 import lib, stencil as S
    u0 = S.init_uniform(shape, SEED)
    host = u0.cpu().numpy()
    a, b = u0.clone(), u0.clone()
    res = S.sweep(a, b, 1, 1000, lib.MODE_JACOBI, "auto")
    engine, launches = S.last_dispatch()
    got = res.cpu().numpy()
    del a, b, res
    torch.cuda.empty_cache()
    assert launches == 1, (engine, launches)
    want = O.run(host.copy(), host.copy(), 1, O.JACOBI, 1000, threads=THREADS)
    assert _bits_equal(got, want), engine
    if len(shape) == 2:
        h64 = host.astype(np.float64)
        r64 = O.run(h64.copy(), h64.copy(), 1, O.JACOBI, 1000, threads=THREADS)
        err = float(np.abs(got - r64).max() / np.abs(r64).max())
        assert err < 1e-6
