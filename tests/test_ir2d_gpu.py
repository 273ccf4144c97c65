"""Mixed-precision refinement on 2-D grids: both engines of stencil_ir_solve
(a launch per correction sweep, and one cooperative launch per outer step
with every sweep in shared memory) bit for bit against the CPU restatement
oracle/ir_oracle.py, and against each other."""
import numpy as np
import pytest

from oracle import ir_oracle as IRO
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _field(shape, seed):
    """Laplace border (smooth, sign-changing) with a uniform [0,1) interior."""
    from thesis_gb300 import stencil as S
    u = S.init_laplace2d(shape, seed)
    noise = S.init_uniform(shape, seed + 1)
    u[1:-1, 1:-1] = noise[1:-1, 1:-1]
    return u


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("storage", ["bf16", "fp16"])
@pytest.mark.parametrize("shape,radius,iters,inner", [
    ((64, 64), 1, 61, 50), ((72, 96), 1, 40, 7), ((130, 200), 2, 33, 16),
    ((96, 64), 4, 25, 9), ((48, 40), 1, 5, 1), ((40, 32), 2, 12, 2), ((512, 512), 1, 300, 100)])
def test_engines_match_oracle(cuda, storage, shape, radius, iters, inner):
    from thesis_gb300 import stencil as S
    u0 = _field(shape, 11 + radius)
    host = u0.cpu().numpy()
    want, outer = IRO.ir_solve(host, radius, iters, inner, storage)
    for engine in ("persistent2d", "launches"):
        u = u0.clone()
        r = S.ir_solve_ex(u, radius, iters, storage, inner_sweeps=inner, engine=engine)
        assert r["engine"] == engine
        assert r["sweeps"] == iters and r["outer_steps"] == outer
        got = u.cpu().numpy()
        bad = int((_bits(got) != _bits(want)).sum())
        assert bad == 0, "%s: %d cells differ from the oracle" % (engine, bad)
    assert S.device_status() == 0


@pytest.mark.parametrize("temporal,tile", [(1, (0, 0)), (3, (16, 8)), (8, (32, 16)), (31, (0, 0)),
                                           (0, (64, 32)), (5, (24, 12))])
def test_persistent_plans_match_oracle(cuda, temporal, tile):
    """Caller-chosen sweeps per exchange and tiles (partial edge tiles included)."""
    from thesis_gb300 import stencil as S
    shape, radius, iters, inner = (136, 120), 1, 45, 20
    u0 = _field(shape, 5)
    want, _ = IRO.ir_solve(u0.cpu().numpy(), radius, iters, inner, "fp16")
    u = u0.clone()
    r = S.ir_solve_ex(u, radius, iters, "fp16", inner_sweeps=inner, engine="persistent2d",
                      temporal=temporal, tile=tile)
    if temporal:
        assert r["temporal"] == min(temporal, inner)
    if tile != (0, 0):
        assert r["tile"] == tile
    assert np.array_equal(_bits(u.cpu().numpy()), _bits(want))
    assert S.device_status() == 0


def test_persistent_matches_launches_full_size(cuda):
    """512^2 R=1 FP16 Laplace problem, 2000 sweeps in steps of 500: the two
    engines agree bit for bit, the border band is untouched, and the result is
    within the FP16 storage precision (unit roundoff 2^-11, relative to the
    field's largest value) of the plain FP32 loop."""
    from thesis_gb300 import stencil as S
    shape = (512, 512)
    u0 = S.init_laplace2d(shape, 21)
    out = {}
    for engine in ("persistent2d", "launches"):
        u = u0.clone()
        S.ir_solve_ex(u, 1, 2000, "fp16", inner_sweeps=500, engine=engine)
        out[engine] = u.cpu().numpy()
    assert np.array_equal(_bits(out["persistent2d"]), _bits(out["launches"]))
    host = u0.cpu().numpy()
    band = np.ones(shape, bool)
    band[1:-1, 1:-1] = False
    assert np.array_equal(_bits(out["persistent2d"][band]), _bits(host[band]))
    fp32 = O.run(host.copy(), host.copy(), 1, O.JACOBI, 2000, threads=8)
    err = float(np.abs(out["persistent2d"] - fp32).max() / np.abs(fp32).max())
    assert err < 2 ** -11


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_persistent_converges_like_launches(cuda, storage):
    """With a tolerance both engines stop after the same outer step and
    return the same grid."""
    from thesis_gb300 import stencil as S
    shape = (256, 256)
    u0 = S.init_laplace2d(shape, 9)
    res = {}
    for engine in ("persistent2d", "launches"):
        u = u0.clone()
        r = S.ir_solve_ex(u, 1, 400000, storage, inner_sweeps=250, tol=1e-5, check_every=1,
                          engine=engine)
        res[engine] = (r, u.cpu().numpy())
    rp, up = res["persistent2d"]
    rl, ul = res["launches"]
    assert rp["rel_residual"] < 1e-5 and rp["sweeps"] < 400000
    assert (rp["sweeps"], rp["outer_steps"]) == (rl["sweeps"], rl["outer_steps"])
    assert rp["rel_residual"] == rl["rel_residual"]
    assert np.array_equal(_bits(up), _bits(ul))
    assert O.rel_residual(up, 1) < 1e-5
    # one cooperative launch per outer step plus the residual checks
    assert rp["kernel_launches"] == rp["outer_steps"] * 3


def test_persistent_rejects_what_it_cannot_run(cuda):
    from thesis_gb300 import lib as L, stencil as S
    u = S.init_laplace2d((4096, 4096), 3)  # more tiles than SMs
    with pytest.raises(L.StencilError) as ei:
        S.ir_solve_ex(u, 1, 10, "fp16", inner_sweeps=5, engine="persistent2d")
    assert ei.value.status == L.EUNSUPPORTED
    # AUTO falls back to the launches on the same grid
    r = S.ir_solve_ex(u, 1, 10, "fp16", inner_sweeps=5)
    assert r["engine"] == "launches"
    v = S.init_fourier((24, 32, 40), 3, 1)
    with pytest.raises(L.StencilError):
        S.ir_solve_ex(v, 1, 10, "fp16", inner_sweeps=5, engine="persistent2d")
