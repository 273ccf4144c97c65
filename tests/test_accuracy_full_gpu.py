"""Full-size accuracy of the benchmark workloads against the oracle: the GPU
result of each headline configuration compared bit for bit with the FP32
oracle (same summation order) and normwise with the FP64 oracle, and the
mixed-precision refinement of the 768^3 R=4 workload against the FP32 run and
the FP64 oracle.

The FP64 oracle at these sizes takes minutes on the host cores (768^3 R=4 x
2000 sweeps is 8.8e11 updates), so the module runs only with
STENCIL_FULL_ACCURACY=1; STENCIL_ACCURACY_OUT names a JSON file for the
numbers.  Inputs are the benchmark's: seed 20251203, uniform [0,1) border and
interior (512^3, 256^2) and an 8-mode Fourier border with uniform interior
(768^3)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.slow,
              pytest.mark.skipif(os.environ.get("STENCIL_FULL_ACCURACY") != "1",
                                 reason="full-size FP64 oracle runs take minutes; "
                                        "set STENCIL_FULL_ACCURACY=1")]

SEED = 20251203
THREADS = len(os.sched_getaffinity(0)) or 8
RESULTS = {}


def _record(key, value):
    RESULTS[key] = value
    out = os.environ.get("STENCIL_ACCURACY_OUT")
    if out:
        with open(out, "w") as f:
            json.dump(RESULTS, f, indent=1)
    print(key, json.dumps(value))


def _normwise(a, ref):
    return float(np.abs(a.astype(np.float64) - ref).max() / np.abs(ref).max())


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("shape,radius,sweeps", [((256, 256), 1, 1000), ((512, 512, 512), 1, 1000),
                                                 ((512, 512, 512), 4, 1000)],
                         ids=["c1_256sq_r1", "c2_512cubed_r1", "c2_512cubed_r4"])
def test_plain_fp32_vs_fp32_and_fp64_oracle(cuda, shape, radius, sweeps):
    import torch
    from thesis_gb300 import stencil as S
    u0 = S.init_uniform(shape, SEED)
    host = u0.cpu().numpy()
    a, b = u0.clone(), u0.clone()
    got = S.sweep(a, b, radius, sweeps, O.JACOBI, "auto").cpu().numpy()
    engine = S.last_dispatch()[0]
    del a, b
    torch.cuda.empty_cache()
    want32 = O.run(host.copy(), host.copy(), radius, O.JACOBI, sweeps, threads=THREADS)
    exact = _bits_equal(got, want32)
    del want32
    h64 = host.astype(np.float64)
    want64 = O.run(h64, h64.copy(), radius, O.JACOBI, sweeps, threads=THREADS)
    err = _normwise(got, want64)
    _record("%s_r%d_%d" % ("x".join(map(str, shape)), radius, sweeps),
            {"engine": engine, "bit_exact_vs_fp32_oracle": exact, "normwise_err_vs_fp64_oracle": err})
    assert exact
    assert err < 1e-5


def test_mixed_precision_768_vs_fp32_and_fp64_oracle(cuda):
    import torch
    from thesis_gb300 import stencil as S
    shape, radius, sweeps = (768, 768, 768), 4, 2000
    u0 = S.init_fourier(shape, SEED, radius, modes=8)
    host = u0.cpu().numpy()
    a, b = u0.clone(), u0.clone()
    fp32 = S.sweep(a, b, radius, sweeps, O.JACOBI, "auto").cpu().numpy()
    del a, b
    torch.cuda.empty_cache()
    irs = {}
    for st in ("bf16", "fp16"):
        u = u0.clone()
        done, outer, rel = S.ir_solve(u, radius, sweeps, st, inner_sweeps=50)
        irs[st] = (u.cpu().numpy(), rel)
        del u
        torch.cuda.empty_cache()
    del u0
    torch.cuda.empty_cache()
    h64 = host.astype(np.float64)
    del host
    want64 = O.run(h64, h64.copy(), radius, O.JACOBI, sweeps, threads=THREADS)
    res = {"fp32": {"normwise_err_vs_fp64_oracle": _normwise(fp32, want64)}}
    for st, (got, rel) in irs.items():
        res["ir_" + st] = {"normwise_err_vs_fp64_oracle": _normwise(got, want64),
                           "normwise_err_vs_fp32": _normwise(got, fp32.astype(np.float64)),
                           "rel_residual": rel}
    _record("768x768x768_r4_2000", res)
    assert res["fp32"]["normwise_err_vs_fp64_oracle"] < 1e-5
    assert res["ir_bf16"]["normwise_err_vs_fp64_oracle"] < 1e-3
    assert res["ir_fp16"]["normwise_err_vs_fp64_oracle"] < 1.5e-4
