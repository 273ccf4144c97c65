"""The reference's HEURISTIC block selection (src/stencil_dispatch.cu:138-146):
the occupancy query with the set_smem sizing, then the shaping rule.

stencil_heuristic_geometry runs the procedure on the kernel this library
launches for the role; oracle/ref_gpu.py runs it, through the driver API, on
the reference's own kernel for the same configuration.  Both must apply the
same rule to their thread counts, and the library's sweeps at its geometry
are bit-exact against the oracle (as is the drop-in binary built with
HEURISTIC=2)."""
import ctypes

import numpy as np
import pytest

from oracle import make_solution as MS
from oracle import oracle as O
from oracle import ref_gpu as RG

pytestmark = pytest.mark.gpu

# (dims, dim, radius, BLOCK_X, BLOCK_Y, BLOCK_Z, COARSEN_X): configurations
# whose reference kernels oracle/build.py compiles
CFGS = [(3, 64, 1, 32, 4, 4, 1), (3, 64, 2, 32, 4, 4, 1), (3, 64, 2, 32, 4, 4, 2),
        (2, 64, 1, 32, 8, 1, 1)]


def _rule(lib, p):
    def shape(threads):
        bx, by, bz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib.check(lib.load().stencil_heuristic_block(ctypes.byref(p), threads, ctypes.byref(bx),
                                                     ctypes.byref(by), ctypes.byref(bz)),
                  "stencil_heuristic_block")
        return bx.value, by.value, bz.value
    return shape


@pytest.mark.parametrize("cfg", CFGS, ids=["%dd_%d_r%d_b%dx%dx%d_cf%d" % c for c in CFGS])
@pytest.mark.parametrize("variant", ["base", "smem", "smem_padded", "smem_register"])
def test_heuristic_geometry_and_results(cuda, cfg, variant):
    from thesis_gb300 import lib, stencil as S
    dims, dim, radius, bx0, by0, bz0, cf = cfg
    shape = (dim,) * dims
    iters = 5
    p = lib.make_params(shape, radius, iters, lib.MODE_JACOBI, variant, (bx0, 0, 0), cf)
    t, bx, by, bz = S.heuristic_geometry(p)
    rule = _rule(lib, p)
    assert t % 32 == 0 and 32 <= t <= 1024
    assert (bx, by, bz) == rule(t)
    if RG.available(cfg):
        ref = RG.RefKernels(cfg)
        try:
            tr, rbx, rby, rbz = ref.heuristic_geometry(variant, rule)
        finally:
            ref.close()
        print("%s %s: library %d threads %s, reference kernel %d threads %s"
              % (cfg, variant, t, (bx, by, bz), tr, (rbx, rby, rbz)))
        assert tr % 32 == 0 and 32 <= tr <= 1024
        if tr == t:
            assert (rbx, rby, rbz) == (bx, by, bz)
    if bz < 1 or by < 1:
        pytest.skip("the rule gives an empty block dimension at %d threads" % t)
    u0 = S.init_uniform(shape, 17)
    host = u0.cpu().numpy()
    block = (bx, by, 0 if (variant == "smem_register" and dims == 3) else bz)
    res = S.sweep(u0.clone(), u0.clone(), radius, iters, lib.MODE_JACOBI, variant,
                  block=block, coarsen_x=cf)
    want = O.run(host.copy(), host.copy(), radius, O.JACOBI, iters, threads=8)
    assert np.array_equal(res.cpu().numpy().view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("variant", [{}, {"SMEM": 1}, {"SMEM": 1, "PADDED": 1},
                                     {"SMEM": 1, "REGISTER": 1}])
def test_dropin_binary_with_reference_heuristic(cuda, tmp_path, variant):
    """constants.h with HEURISTIC=2: the drop-in binary takes the reference's
    occupancy-based block and passes its DEBUG known-answer check."""
    import subprocess
    from thesis_gb300 import build as B
    cfg = {"DIM": 48, "DIMENSIONS": 3, "RADIUS": 2, "ITERATIONS": 8, "DEBUG": 1, "HEURISTIC": 2}
    MS.write_solution(48, 3, 2, 8, str(tmp_path))
    exe = B.build_main({**cfg, **variant}, out=str(tmp_path / "stencil_bin"))
    res = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "rms error = 0.000000" in res.stdout
