"""bench.py's replica path (N > 1: one independent replica per GPU, no data
exchange) on the host: world size 2 over gloo on 127.0.0.1.  The step time is
the slowest rank's, the reported rate is the whole job's, and the reference
arm runs on rank 0 alone."""
import importlib.util
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        b = _bench()
        # each rank's own step time; rank 1 is the slow replica
        mine = 0.25 + 0.5 * rank
        q.put((rank, b.max_over_ranks(mine, world, "cpu")))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 0.75, 1: 0.75}


def test_whole_job_rate_and_single_rank():
    b = _bench()
    assert b.max_over_ranks(1.5, 1, None) == 1.5
    # two replicas of 10 steps of 1e9 updates in 4 s: 5 GCell-updates/s for the job
    assert b.aggregate_rate(1e9, 10, 2, 4.0) == pytest.approx(5.0)
    assert b.aggregate_rate(1e9, 10, 1, 4.0) == pytest.approx(2.5)


def test_reference_arm_runs_on_rank_0_only(monkeypatch, capsys):
    b = _bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    b.run_reference(b.parse())
    assert capsys.readouterr().out == ""


def test_reference_arm_json_contract(monkeypatch, capsys):
    """bench.py --impl reference on rank 0: one JSON line with the metric of
    the GPU arm, the CPU baseline it measured and an e2e block without host
    copies (a small grid here; each step is a bounded sample of about 8 s)."""
    import json
    b = _bench()
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--dim", "48",
                                      "--steps", "1", "--warmup", "0"])
    b.run_reference(b.parse())
    line = capsys.readouterr().out.strip().splitlines()[-1]
    d = json.loads(line)
    assert d["impl"] == "reference"
    assert d["unit"] == "GCell-updates/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["metric"].startswith("GCell-updates/s")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["dim"] == 48 and d["config"]["radius"] == 1
