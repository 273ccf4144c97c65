"""The reference-facing edges of the path: the drop-in binary (ms as the last
stdout line, DEBUG known-answer check, src/main.cu:10-103), the known-answer
solution files (include/stencil_utils.h:16-76) and the results-JSON harness
(scripts/evaluate_stencils.py)."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import make_solution as MS
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name,dim,dims,radius,iters", [
    ("legacy_3d_64_r2_i8.npz", 64, 3, 2, 8), ("legacy_2d_67_r3_i8.npz", 67, 2, 3, 8),
    ("legacy_2d_64_r1_i7.npz", 64, 2, 1, 7)])
def test_solution_file_is_the_reference_output(tmp_path, name, dim, dims, radius, iters):
    """The known-answer file equals the reference's own stencil_cpu output."""
    want = np.load(os.path.join(GOLDEN, name))["grid"]
    path = MS.write_solution(dim, dims, radius, iters, str(tmp_path))
    assert os.path.basename(path) == "solution_%d_%d_%d_%dd" % (dim, iters, radius, dims)
    got = np.fromfile(path, np.float32).reshape(want.shape)
    assert np.array_equal(got.view(np.uint32), np.ascontiguousarray(want, np.float32).view(np.uint32))


def test_dropin_binary_builds(tmp_path):
    from thesis_gb300 import build as B
    for d in ({"DIM": 32, "DIMENSIONS": 3, "RADIUS": 1, "ITERATIONS": 8},
              {"DIM": 64, "DIMENSIONS": 2, "RADIUS": 4, "ITERATIONS": 3, "SMEM": 1, "PADDED": 1,
               "HEURISTIC": 0, "BLOCK_X": 32, "BLOCK_Y": 8, "BLOCK_Z": 1, "DEBUG": 1}):
        exe = B.build_main(d, out=str(tmp_path / "stencil_test"))
        assert os.access(exe, os.X_OK)


def test_results_schema_and_resume(tmp_path, monkeypatch):
    from thesis_gb300 import evaluate as E
    calls = []

    def fake(dimensions, dim, version, radius, iterations, unroll, block, repeat, mode):
        calls.append((dimensions, dim, version, radius, iterations, unroll, block))
        return [1.5] * repeat

    monkeypatch.setattr(E, "run_inprocess", fake)
    out = str(tmp_path / "results" / "results_stencils.json")
    tune = tmp_path / "results" / "results_autotune.json"
    os.makedirs(tune.parent, exist_ok=True)
    tune.write_text(json.dumps({"3": {"32": {"smem_unroll_2": {"4": {"BLOCK_X": 64, "BLOCK_Y": 4,
                                                                     "BLOCK_Z": 2}}}}}))
    E.evaluate([3], [32], ["base", "smem"], [1, 4], [1, 2], [8], host="h", repeat=3, out=out,
               log=None)
    assert len(calls) == 8
    db = json.load(open(out))
    assert db["3"]["32"]["1_gpus_base"]["1"]["8"]["h"]["heuristic"]["time"] == [1.5] * 3
    assert "1_gpus_smem_unroll_2" in db["3"]["32"]
    # resume: every entry exists, nothing runs again
    E.evaluate([3], [32], ["base", "smem"], [1, 4], [1, 2], [8], host="h", repeat=3, out=out,
               log=None)
    assert len(calls) == 8
    # autotune: the block shape comes from the tuning database
    E.evaluate([3], [32], ["smem"], [4], [2], [8], host="h", autotune=True, repeat=2, out=out,
               tune_path=str(tune), log=None)
    assert calls[-1][-1] == (64, 4, 2)
    assert "autotune" in json.load(open(out))["3"]["32"]["1_gpus_smem_unroll_2"]["4"]["8"]["h"]


# ---------------------------------------------------------------- GPU -----

CFG = {"DIM": 48, "DIMENSIONS": 3, "RADIUS": 2, "ITERATIONS": 8, "DEBUG": 1}


def _run(exe, cwd):
    return subprocess.run([exe], cwd=cwd, capture_output=True, text=True, timeout=300)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [{}, {"SMEM": 1}, {"SMEM": 1, "PADDED": 1},
                                     {"SMEM": 1, "REGISTER": 1}, {"COOP": 1}])
def test_dropin_binary_debug_check(cuda, tmp_path, variant):
    from thesis_gb300 import build as B
    MS.write_solution(48, 3, 2, 8, str(tmp_path))
    exe = B.build_main({**CFG, **variant}, out=str(tmp_path / "stencil_bin"))
    res = _run(exe, tmp_path)
    assert res.returncode == 0, res.stdout + res.stderr
    lines = res.stdout.strip().splitlines()
    assert "rms error = 0.000000" in res.stdout
    assert float(lines[-1]) > 0.0


@pytest.mark.gpu
def test_dropin_binary_rejects_wrong_or_missing_answer(cuda, tmp_path):
    from thesis_gb300 import build as B
    exe = B.build_main(CFG, out=str(tmp_path / "stencil_bin"))
    res = _run(exe, tmp_path)
    assert res.returncode != 0 and "Unable to load file" in res.stdout
    path = MS.write_solution(48, 3, 2, 8, str(tmp_path))
    grid = np.fromfile(path, np.float32)
    grid[48 * 48 * 20 + 48 * 20 + 20] += 0.01
    grid.tofile(path)
    res = _run(exe, tmp_path)
    assert res.returncode != 0
    grid[5] = np.nan
    grid.tofile(path)
    assert _run(exe, tmp_path).returncode != 0


@pytest.mark.gpu
def test_results_json_through_library_and_binary(cuda, tmp_path):
    from thesis_gb300 import evaluate as E
    for binary in (False, True):
        out = str(tmp_path / ("b" if binary else "l") / "results.json")
        E.evaluate([3], [32], ["base", "smem_register"], [1], [1], [8], host="gb300", repeat=2,
                   out=out, binary=binary, log=None)
        db = json.load(open(out))
        for v in ("1_gpus_base", "1_gpus_smem_register"):
            t = db["3"]["32"][v]["1"]["8"]["gb300"]["heuristic"]["time"]
            assert len(t) == 2 and all(x > 0 for x in t)


@pytest.mark.gpu
def test_timed_host_run_splits_sweeps(cuda):
    from thesis_gb300 import stencil as S
    u = O.uniform((40, 40, 64), seed=4)
    out, ms, ms_sw = S.run_host(u, 1, 6, O.JACOBI, sweeps_ms=True)
    assert 0 < ms_sw <= ms
    a, b = u.copy(), u.copy()
    want = O.run(a, b, 1, O.JACOBI, 6)
    assert np.array_equal(out.view(np.uint32), want.view(np.uint32))
