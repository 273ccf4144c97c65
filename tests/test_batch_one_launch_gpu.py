"""GPU parity of the one-launch batch engine (every grid of a batch in ONE
persistent cooperative launch: teams of CTAs take grids from device queues,
tier by tier), bit for bit against the oracle, with CUDA-graph replays."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def oracle_pair(u, radius, iters, mode):
    a, b = u.copy(), u.copy()
    res = O.run(a, b, radius, mode, iters, threads=8)
    return res, (b if res is a else a)


# 2-D and 3-D, R = 1..4, JACOBI and LEGACY, ragged widths (swept in pitched
# copies staged inside the launch), 0 and 1 sweeps, grids from a few cells
# to a few million (teams of one CTA up to a quarter of the GPU).
SPECS = [
    ((64, 64), 1, 12, "jacobi"),
    ((70, 66), 1, 23, "jacobi"),          # ragged
    ((131, 127), 2, 9, "jacobi"),         # ragged
    ((40, 36), 3, 6, "legacy"),
    ((64, 64), 4, 5, "jacobi"),
    ((9, 13), 4, 3, "jacobi"),            # the smallest 2-D grid at R = 4, ragged
    ((200, 256), 1, 0, "jacobi"),         # no sweep: the result is d_u1 as given
    ((256, 200), 2, 1, "legacy"),
    ((1024, 1024), 1, 6, "jacobi"),
    ((1500, 1301), 1, 5, "jacobi"),       # ragged
    ((900, 640), 2, 5, "jacobi"),
    ((700, 620), 4, 4, "legacy"),
    ((30, 32, 32), 1, 12, "jacobi"),
    ((37, 41, 43), 2, 11, "jacobi"),      # ragged
    ((24, 20, 24), 2, 5, "legacy"),
    ((20, 22, 26), 3, 4, "jacobi"),       # ragged
    ((17, 18, 20), 4, 3, "jacobi"),
    ((9, 9, 9), 4, 2, "jacobi"),          # the smallest 3-D grid at R = 4, ragged
    ((96, 96, 96), 2, 4, "jacobi"),
    ((120, 120, 120), 1, 9, "jacobi"),
    ((150, 131, 141), 2, 7, "jacobi"),    # ragged
    ((128, 128, 128), 1, 4, "legacy"),
    ((160, 144, 128), 2, 6, "jacobi"),
    ((100, 90, 88), 3, 3, "jacobi"),
    ((96, 80, 72), 4, 3, "legacy"),
]


def _make(specs, seed0):
    import torch
    hosts, jobs, modes = [], [], []
    for k, (shape, radius, iters, mode) in enumerate(specs):
        u = O.uniform(shape, seed=seed0 + k)
        m = O.JACOBI if mode == "jacobi" else O.LEGACY
        hosts.append(u)
        modes.append(m)
        jobs.append((torch.from_numpy(u).cuda(), torch.from_numpy(u).cuda(), radius, iters, m))
    return hosts, jobs, modes


def _wants(specs, hosts, modes):
    out = []
    for k, (shape, radius, iters, _) in enumerate(specs):
        out.append(oracle_pair(hosts[k], radius, iters, modes[k]))
    return out


def _check(b, specs, wants, jobs):
    for k, (shape, radius, iters, _) in enumerate(specs):
        want, other = wants[k]
        res = b.result(k)
        oth = jobs[k][1] if res is jobs[k][0] else jobs[k][0]
        assert bits_equal(res.cpu().numpy(), want), (k, shape, radius, iters)
        # the other buffer holds what the ping-pong loop leaves there
        assert bits_equal(oth.cpu().numpy(), other), ("other buffer", k, shape, radius, iters)


def _reset(jobs, hosts):
    import torch
    for k in range(len(jobs)):
        jobs[k][0].copy_(torch.from_numpy(hosts[k]))
        jobs[k][1].copy_(torch.from_numpy(hosts[k]))
    torch.cuda.synchronize()


# (STENCIL_BATCH1_CELLS_PER_CTA_2D, _3D, STENCIL_BATCH1_MAX_TEAM): the
# defaults; every grid on a team of one CTA; every grid on the largest team
# allowed; many tiers with small teams and remainders.
TEAMS = [("", "", ""), ("1000000000", "1000000000", ""), ("1", "1", ""), ("5000", "7000", "16"),
         ("", "", "1")]


@pytest.mark.parametrize("cpc2,cpc3,maxteam", TEAMS)
def test_one_launch_batch_matches_oracle_and_graph_replay(cuda, monkeypatch, cpc2, cpc3, maxteam):
    import torch
    from thesis_gb300 import stencil as S
    monkeypatch.setenv("STENCIL_BATCH1_CELLS_PER_CTA_2D", cpc2)
    monkeypatch.setenv("STENCIL_BATCH1_CELLS_PER_CTA_3D", cpc3)
    monkeypatch.setenv("STENCIL_BATCH1_MAX_TEAM", maxteam)
    hosts, jobs, modes = _make(SPECS, 500)
    b = S.Batch(jobs, engine="one_launch")
    assert b.kernel_launches() == 1
    assert b.plan() == (0, 0)
    tiers = b.teams()
    assert sum(n for _, n in tiers) == len(SPECS)
    assert all(t1 > t2 for (t1, _), (t2, _) in zip(tiers, tiers[1:]))  # largest teams first
    if maxteam == "1" or cpc2 == "1000000000":
        assert tiers == [(1, len(SPECS))]
    b.launch()
    torch.cuda.synchronize()
    wants = _wants(SPECS, hosts, modes)
    _check(b, SPECS, wants, jobs)
    # captured into a CUDA graph (a memset node and one kernel node), replayed
    # twice from reset inputs: the queues and team counters start afresh
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            b.launch(stream=s)
    for _ in range(2):
        _reset(jobs, hosts)
        g.replay()
        torch.cuda.synchronize()
        _check(b, SPECS, wants, jobs)
    b.close()
    assert S.device_status() == 0


def test_one_launch_batch_engines_agree_on_benchmark_like_mix(cuda):
    """A scaled-down mix of the 512-grid benchmark batch (2-D R = 1 sides
    log-uniform, 3-D R = 2 sides log-uniform, sweeps uniform): both engines
    give bit-identical results, and the one-launch result matches the oracle
    on a sample."""
    import torch
    from thesis_gb300 import stencil as S
    rng = np.random.default_rng(77)
    specs = []
    for _ in range(40):
        n = int(round(np.exp(rng.uniform(np.log(64), np.log(1024)))))
        specs.append(((n, n), 1, int(rng.integers(1, 40)), "jacobi"))
    for _ in range(12):
        n = int(round(np.exp(rng.uniform(np.log(32), np.log(160)))))
        specs.append(((n, n, n), 2, int(rng.integers(1, 20)), "jacobi"))
    hosts, jobs1, modes = _make(specs, 900)
    _, jobs2, _ = _make(specs, 900)
    b1 = S.Batch(jobs1, engine="one_launch")
    b2 = S.Batch(jobs2, engine="phased")
    b1.launch()
    b2.launch()
    torch.cuda.synchronize()
    for k in range(len(specs)):
        assert bits_equal(b1.result(k).cpu().numpy(), b2.result(k).cpu().numpy()), (k, specs[k])
    for k in range(0, len(specs), 5):
        want, _ = oracle_pair(hosts[k], specs[k][1], specs[k][2], modes[k])
        assert bits_equal(b1.result(k).cpu().numpy(), want), (k, specs[k])
    b1.close()
    b2.close()
    assert S.device_status() == 0


def test_one_launch_batch_reprepare_and_env_engine(cuda, monkeypatch):
    """STENCIL_BATCH_ENGINE=one_launch makes "auto" the one-launch engine; a
    workspace prepared again with the other engine follows the new plan."""
    import torch
    from thesis_gb300 import lib as L
    from thesis_gb300 import stencil as S
    specs = SPECS[:6] + SPECS[12:16]
    hosts, jobs, modes = _make(specs, 700)
    monkeypatch.setenv("STENCIL_BATCH_ENGINE", "one_launch")
    b = S.Batch(jobs)
    assert b.kernel_launches() == 1 and b.teams()
    monkeypatch.setenv("STENCIL_BATCH_ENGINE", "phased")
    b2 = S.Batch(jobs)
    assert b2.teams() == []
    b.launch()
    torch.cuda.synchronize()
    _check(b, specs, _wants(specs, hosts, modes), jobs)
    b.close()
    b2.close()
    lib = L.load()
    rc = lib.stencil_batch_prepare_engine(None, 0, 3, 0, b.workspace.data_ptr(), 0, None)
    assert rc == L.EINVAL
    # an empty batch: nothing to launch
    monkeypatch.delenv("STENCIL_BATCH_ENGINE")
    e = S.Batch([], engine="one_launch")
    assert e.kernel_launches() == 0 and e.teams() == []
    e.launch()
    torch.cuda.synchronize()
    e.close()


def test_one_launch_team_tuner_and_tuned_batch_match_oracle(cuda):
    """The team-size tuner on a copy of the batch, then the batch with its
    team fields (AUTO still picks the one-launch engine for team-only hints):
    bit-exact against the oracle; a team field beyond the device's CTAs is
    clamped."""
    import torch
    from thesis_gb300 import autotune as A
    from thesis_gb300 import stencil as S
    specs = [((96, 100), 1, 9, "jacobi"), ((301, 257), 1, 7, "jacobi"), ((700, 720), 1, 5, "jacobi"),
             ((1030, 1024), 1, 4, "jacobi"), ((40, 36, 44), 2, 6, "jacobi"), ((64, 64, 64), 2, 5, "jacobi"),
             ((120, 112, 108), 2, 4, "jacobi"), ((130, 128, 126), 2, 3, "jacobi")]
    hosts, jobs, modes = _make(specs, 1300)

    def make():
        return [(j[0].clone(), j[1].clone()) + tuple(j[2:]) for j in jobs]

    tuned = A.tune_batch_teams(make, log=None)
    assert set(tuned) == {"2d_small", "2d_large", "3d_small", "3d_large"}
    for r in tuned.values():
        assert r["choice"]["cells_per_cta"] in A.BATCH1_SPACE["2d_small"]["cells_per_cta"]
        assert r["s"] < float("inf") and r["default_s"] < float("inf")
    b = S.Batch(jobs, hints_for=A.batch_team_hints({"batch_one_launch": tuned}))
    assert b.kernel_launches() == 1 and b.teams()
    b.launch()
    torch.cuda.synchronize()
    _check(b, specs, _wants(specs, hosts, modes), jobs)
    b.close()
    # a team field larger than the device's CTA count is clamped to it
    _reset(jobs, hosts)
    b = S.Batch([j + ({"team": 100000},) for j in jobs], engine="one_launch")
    assert max(t for t, _ in b.teams()) <= torch.cuda.get_device_properties(0).multi_processor_count * 8
    b.launch()
    torch.cuda.synchronize()
    _check(b, specs, _wants(specs, hosts, modes), jobs)
    b.close()
    assert S.device_status() == 0


def test_one_launch_batch_zero_sweep_grids_keep_teams_together(cuda, monkeypatch):
    """Grids with no sweep between swept ones, all on large teams: every team
    stays on one grid at a time (a zero-sweep grid ends with a team barrier),
    over several CUDA-graph replays."""
    import torch
    from thesis_gb300 import stencil as S
    monkeypatch.setenv("STENCIL_BATCH1_CELLS_PER_CTA_2D", "1")
    monkeypatch.setenv("STENCIL_BATCH1_CELLS_PER_CTA_3D", "1")
    specs = []
    for k in range(24):
        if k % 2:
            specs.append(((64 + 8 * k, 60 + 4 * k), 1, 0, "jacobi"))
        elif k % 4 == 0:
            specs.append(((40 + k, 36, 44), 2, 3 + k % 5, "jacobi"))
        else:
            specs.append(((300 + 10 * k, 257), 1, 2 + k % 7, "jacobi"))
    hosts, jobs, modes = _make(specs, 1700)
    b = S.Batch(jobs, engine="one_launch")
    wants = _wants(specs, hosts, modes)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        b.launch(stream=s)
        s.synchronize()
        with torch.cuda.graph(g, stream=s):
            b.launch(stream=s)
    for _ in range(4):
        _reset(jobs, hosts)
        g.replay()
        torch.cuda.synchronize()
        _check(b, specs, wants, jobs)
    b.close()
    assert S.device_status() == 0


def test_one_launch_matches_phased_on_the_benchmark_batch(cuda):
    """The 512-grid benchmark batch at full size (384 2-D R=1 grids of
    64..2048, 128 3-D R=2 grids of 32..256, 100..5000 sweeps; 382 ragged
    widths): the one-launch engine's results equal the phased engine's bit
    for bit in every grid (the phased engine is pinned to the oracle above
    and in test_cluster_gpu.py), with its default and with tuned-looking
    team sizes."""
    import torch
    from bench import c4_jobs
    from thesis_gb300 import lib as L
    from thesis_gb300 import stencil as S
    specs = c4_jobs()
    init = [S.init_uniform(sp[0], 31 + k) for k, sp in enumerate(specs)]
    outs = {}
    for name, engine, hints in [("phased", "phased", None), ("one", "one_launch", None),
                                ("one_teams", "one_launch", lambda shape: {"team": 38 if len(shape) == 3 else 9})]:
        jobs = [(u.clone(), u.clone(), sp[1], sp[2], L.MODE_JACOBI) for u, sp in zip(init, specs)]
        b = S.Batch(jobs, engine=engine, hints_for=hints)
        b.launch()
        torch.cuda.synchronize()
        outs[name] = [b.result(k) for k in range(len(jobs))]
        b.close()
    for name in ("one", "one_teams"):
        bad = [k for k in range(len(specs))
               if not torch.equal(outs[name][k].view(torch.int32), outs["phased"][k].view(torch.int32))]
        assert not bad, (name, bad[:5], [specs[k] for k in bad[:5]])
    assert S.device_status() == 0
