"""The batch's tuning fields (stencil_batch_job temporal / tile_x / tile_y)
and the autotuner that chooses them per class of grid: every choice is
bit-exact against the oracle, and the tuner's database entry is what Batch
applies."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _jobs(specs, seed=5):
    from thesis_gb300 import stencil as S
    out = []
    for k, (shape, R, it) in enumerate(specs):
        u = S.init_uniform(shape, seed + k)
        out.append((u, u.clone(), R, it, O.JACOBI))
    return out


def _check(bt, jobs, hosts):
    for k, (u1, u2, R, it, mode) in enumerate(jobs):
        want = O.run(hosts[k].copy(), hosts[k].copy(), R, mode, it, threads=8)
        got = bt.result(k).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (k, u1.shape, R, it)


# (shape, R, sweeps) per class, with hints that exercise each field
CASES = [
    ([((96, 128), 1, 37), ((200, 160), 2, 20)], {"temporal": 8}),          # 2d_small, tblock 8
    ([((72, 64), 1, 9)], {"temporal": 1}),                                   # 2d_small, tblock 1
    ([((40, 48, 64), 2, 11), ((56, 56, 56), 1, 6)], {"temporal": 8}),       # 3d_small
    ([((720, 704), 1, 33)], {"temporal": 6, "tile": (64, 32)}),             # 2d_large, tb2d hints
    ([((160, 128, 136), 1, 9), ((130, 120, 128), 2, 7)], {"temporal": 2}),  # 3d_large, tb3d
    ([((150, 128, 128), 2, 8)], {"temporal": 3}),                            # 3d_large, tb3d T=3
    # hints tuned on a smaller grid of the class that do not fit this one
    # (no tile of depth 16 fits one tile per SM): the library's plan runs
    ([((1400, 1502), 1, 21)], {"temporal": 16, "tile": (16, 4)}),           # 2d_large, ragged
]


@pytest.mark.parametrize("specs,hint", CASES)
def test_batch_hints_bit_exact(cuda, specs, hint):
    from thesis_gb300 import stencil as S
    jobs = _jobs(specs)
    hosts = [j[0].cpu().numpy() for j in jobs]
    bt = S.Batch([j + (hint,) for j in jobs], engine="phased")
    bt.launch()
    _check(bt, jobs, hosts)
    bt.close()
    assert S.device_status() == 0


def test_batch_rejects_bad_hints(cuda):
    from thesis_gb300 import lib as L, stencil as S
    jobs = _jobs([((64, 64), 1, 4)])
    with pytest.raises(L.StencilError):
        S.Batch([jobs[0] + ({"temporal": -1},)])
    with pytest.raises(L.StencilError):
        S.Batch([jobs[0] + ({"tile": (30, 16)},)])


def test_tune_batch_and_apply(cuda):
    """The tuner on a small proxy of two classes; the chosen hints, applied
    through the database, give oracle-exact results."""
    from thesis_gb300 import autotune as A, stencil as S
    specs = {"2d_small": [((128, 128), 1, 60), ((96, 96), 1, 40)],
             "3d_large": [((128, 128, 128), 1, 12)]}
    res = A.tune_batch(lambda c: _jobs(specs.get(c, [])), classes=list(specs), repeats=1, log=None)
    assert set(res) == set(specs)
    for c, r in res.items():
        assert r["s"] <= r["default_s"] and r["s"] > 0
    db = {"batch": res}
    jobs = _jobs(specs["2d_small"] + specs["3d_large"], seed=9)
    hosts = [j[0].cpu().numpy() for j in jobs]
    bt = S.Batch(jobs, hints_for=A.batch_hints(db), engine="phased")
    bt.launch()
    _check(bt, jobs, hosts)
    bt.close()
