"""The project's autotuner: search space, optimiser (against brute force on
synthetic scores, as the reference tuner's own self-tests did with fake
evaluators), the JSON database and the library's tuning table."""
import ctypes
import itertools
import json
import os
import tempfile

import pytest

from thesis_gb300 import autotune as A
from thesis_gb300 import lib as L


def test_block_filter_matches_reference_constraints():
    shapes = A.block_shapes(3)
    assert (32, 2, 2) in shapes and (32, 8, 4) in shapes  # reference defaults / heuristic
    for bx, by, bz in shapes:
        assert 32 <= bx * by * bz <= 1024 and bx >= by >= bz and bx >= 8
    assert all(bz == 1 for _, _, bz in A.block_shapes(2))


def test_coordinate_descent_finds_separable_optimum():
    space = {"a": list(range(6)), "b": list(range(5)), "c": [1, 2, 4, 8]}
    target = {"a": 4, "b": 1, "c": 8}
    score = lambda cfg: sum((cfg[k] - target[k]) ** 2 for k in target) + 1.0
    best, s, n = A.coordinate_descent({"a": 0, "b": 0, "c": 1}, space, score)
    brute = min((dict(zip(space, v)) for v in itertools.product(*space.values())), key=score)
    assert best == brute == target and s == 1.0
    assert n < 6 * 5 * 4  # fewer evaluations than brute force


def test_optimise_picks_variant_then_its_parameters():
    top = [{"variant": "x"}, {"variant": "y", "k": 3}]
    sub = {"y": {"k": [1, 2, 3, 4, 5]}}
    score = lambda c: 10.0 if c["variant"] == "x" else abs(c["k"] - 2) + 1.0
    best, s, _ = A.optimise(top, sub, score)
    assert best == {"variant": "y", "k": 2} and s == 1.0


def test_infinite_score_is_never_chosen():
    top = [{"variant": "broken"}, {"variant": "ok"}]
    best, s, _ = A.optimise(top, {}, lambda c: float("inf") if c["variant"] == "broken" else 2.0)
    assert best["variant"] == "ok"


def test_tuning_table_and_db_round_trip(stencil_lib):
    stencil_lib.stencil_tuning_clear()
    entry = {"dims": 3, "radius": 1, "shape": [100, 100, 96], "bucket": 128,
             "choice": {"variant": "smem_padded", "block": [32, 4, 2], "coarsen_x": 8}}
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "db.json")
        A.save_db(path, [entry], "test")
        A.load_db(path)
    key = L.make_params((120, 128, 128), 1, 0)  # same (dims, radius, bucket 128)
    out = L.StencilParams()
    assert stencil_lib.stencil_tuning_get(ctypes.byref(key), ctypes.byref(out)) == 0
    assert out.variant == L.VARIANT_SMEM_PADDED and (out.block_x, out.block_y, out.block_z) == (32, 4, 2)
    assert out.coarsen_x == 8
    other = L.make_params((300, 300, 300), 1, 0)  # bucket 512: no entry
    assert stencil_lib.stencil_tuning_get(ctypes.byref(other), ctypes.byref(out)) == L.EINVAL
    stencil_lib.stencil_tuning_clear()
    assert stencil_lib.stencil_tuning_get(ctypes.byref(key), ctypes.byref(out)) == L.EINVAL


@pytest.mark.gpu
def test_tune_on_gpu_and_auto_uses_it(cuda):
    import numpy as np
    import torch
    from thesis_gb300 import stencil as S
    entry = A.tune((64, 64, 128), 1, sweeps=5, repeats=1, log=None)
    assert entry["us_per_sweep"] > 0 and entry["candidates"] >= 3
    A.install(entry)
    u = S.init_uniform((64, 64, 128), 3)
    got = S.sweep(u.clone(), u.clone(), 1, 7, L.MODE_JACOBI, "auto").cpu().numpy()
    want = S.sweep(u.clone(), u.clone(), 1, 7, L.MODE_JACOBI, "base").cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    L.load().stencil_tuning_clear()


def test_search_space_covers_3d_temporal_blocking_and_batch_classes():
    top, sub = A.variant_space((256, 256, 256), 1)
    assert {"variant": "coop"} in top and sub["coop"]["temporal"] == [0, 2, 3, 4]
    _, sub4 = A.variant_space((256, 256, 256), 4)
    assert sub4["coop"]["temporal"] == [0]  # temporal blocking needs R <= 2
    assert A.batch_class((128, 128)) == "2d_small" and A.batch_class((2048, 2048)) == "2d_large"
    assert A.batch_class((96, 96, 96)) == "3d_small" and A.batch_class((200, 200, 200)) == "3d_large"
    assert set(A.BATCH_SPACE) == {"2d_small", "2d_large", "3d_small", "3d_large"}
    db = {"batch": {"3d_large": {"choice": {"temporal": 2, "tile": [0, 0]}}}}
    hints = A.batch_hints(db)
    assert hints((200, 200, 200)) == {"temporal": 2, "tile": [0, 0]}
    assert hints((64, 64)) is None and A.batch_hints({})((64, 64)) is None


def test_team_tuner_picks_fastest_and_rejects_changed_results():
    """The one-launch engine's team tuner over BATCH1_SPACE with a stand-in
    timer: coordinate descent over the classes present in the proxy batch
    finds the fastest combination, a candidate whose results differ in a bit
    from the default's is rejected, and the database section maps every grid
    of a class to its team field."""
    import torch
    jobs = [(torch.zeros(1000, 1000), torch.zeros(1000, 1000), 1, 10, 1),   # 2d_large
            (torch.zeros(100, 100), torch.zeros(100, 100), 1, 7, 1)]        # 2d_small
    seen = []

    def fake(hinted):
        big, small = (h[5]["team"] for h in hinted)
        seen.append((big, small))
        # 1e6 cells: 12500 -> 80, 25000 -> 40, 50000 -> 20, 100000 -> 10, 200000 -> 5
        t = {80: 5.0, 40: 1.0, 20: 4.0, 10: 2.0, 5: 3.0}[big] + (0.0 if small == 1 else 0.5)
        res = [torch.ones(3), torch.ones(2)]
        if big == 40:
            res = [torch.full((3,), 2.0), torch.ones(2)]  # a candidate that changes a result
        return t, res

    out = A.tune_batch_teams(lambda: [tuple(j) for j in jobs], time_batch=fake, log=None)
    assert set(out) == {"2d_large", "2d_small"}
    assert out["2d_large"]["choice"] == {"cells_per_cta": 100000}   # 40 is faster but wrong
    assert out["2d_small"]["choice"]["cells_per_cta"] >= 12500       # 10^4 cells: team 1 for all
    assert out["2d_large"]["default_s"] == 4.0 and out["2d_large"]["s"] == 2.0
    assert {b for b, _ in seen} == {80, 40, 20, 10, 5}
    hints = A.batch_team_hints({"batch_one_launch": out})
    assert hints((2000, 2000)) == {"team": 40} and hints((64, 64, 64)) is None
    assert A.team_for((10, 10, 10), 50000) == 1 and A.team_for((200, 200, 200), 50000) == 160


def test_coordinate_descent_min_gain_keeps_the_start_within_noise():
    space = {"a": [1, 2, 3]}
    score = {1: 1.0, 2: 0.995, 3: 0.98}
    best, s, _ = A.coordinate_descent({"a": 1}, space, lambda c: score[c["a"]], min_gain=0.01)
    assert best == {"a": 3} and s == 0.98          # 2 % better: taken
    score[3] = 0.995
    best, s, _ = A.coordinate_descent({"a": 1}, space, lambda c: score[c["a"]], min_gain=0.01)
    assert best == {"a": 1} and s == 1.0           # 0.5 %: noise, the start stays
