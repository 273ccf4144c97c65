"""CPU emulation of the one-launch batch kernel's control protocol
(thesis_gb300/csrc/k_batch1.cu): CTAs as coroutines stepped in random order
over shared counters, mailboxes and queues, following the kernel's steps --
team split per tier, the leader's queue atomic and mailbox word, team
barriers (release add, acquire spin), the 3-D sweep barrier that only the
first min(items, team) CTAs join, the 2-D per-sweep team barrier, the copies
of ragged grids.  Checks, under many interleavings: every grid is swept once,
by all the CTAs of one team; no CTA starts sweep s of a grid before every
CTA that sweeps it finished sweep s-1; copies out only after the last sweep;
no deadlock.  Two planted mistakes (idle CTAs joining the sweep barrier; a
grid with no sweep ending without a team barrier, which this emulation found
in the kernel) must be caught."""
import random

import pytest

STOP = -1


def split(start, size, k, cta):
    kk = max(1, k)
    n = max(1, size // kk)
    idx = min((cta - start) // kk, n - 1)
    start += idx * kk
    size = size - idx * kk if idx == n - 1 else kk
    return start, size


class Shared:
    def __init__(self, ntiers, grid):
        self.queue = [0] * ntiers
        self.tbar = {}
        self.sbar = {}
        self.mail = {}
        self.log = []  # (event, job, cta, sweep)


def cta_program(cta, grid, tiers, jobs, sh, plant_idle_arrivals=False, skip_empty_barrier=False):
    """Yields while it waits; appends its sweep events to sh.log."""
    t, start, size, rel, cnt, scnt, job = -1, 0, grid, 0, 0, 0, STOP

    def barrier(key):
        nonlocal cnt
        sh.tbar[key] = sh.tbar.get(key, 0) + 1
        cnt += size
        while sh.tbar[key] < cnt:
            yield

    while True:
        # next_job (thread 0)
        while True:
            if t < 0 or job == STOP:
                t += 1
                if t >= len(tiers):
                    return
                start, size = split(start, size, tiers[t]["team"], cta)
                rel, cnt, scnt = cta - start, 0, 0
            key = (t, start)
            if rel == 0:
                j = sh.queue[t]
                sh.queue[t] += 1
                sh.mail[key] = j
                yield
            yield from barrier(key)
            yield  # the mailbox is read some time after the wait ends
            j = sh.mail[key]
            if j < tiers[t]["njobs"]:
                job = tiers[t]["first"] + j
                break
            job = STOP
        J = jobs[job]
        key = (t, start)
        if J["iters"] <= 0:
            # no sweep, but the team barrier: the leader's next mailbox
            # write must follow every member's read of this index
            if not skip_empty_barrier:
                yield from barrier(key)
            continue
        if J["staged"]:
            sh.log.append(("stage_in", job, cta, -1))
            yield from barrier(key)
        if J["dims"] == 3:
            P = min(J["items"], size)
            joins = rel < P or plant_idle_arrivals
            if joins:
                for sw in range(J["iters"]):
                    if rel < P:
                        # the producer waits for every participant's arrival of the previous sweeps
                        while sw > 0 and sh.sbar.get(key, 0) < scnt + sw * P:
                            yield
                        sh.log.append(("start", job, cta, sw))
                        yield
                        sh.log.append(("end", job, cta, sw))
                    if sw + 1 < J["iters"]:
                        sh.sbar[key] = sh.sbar.get(key, 0) + 1
                        yield
            scnt += (J["iters"] - 1) * P
        else:
            for sw in range(J["iters"]):
                sh.log.append(("start", job, cta, sw))
                yield
                sh.log.append(("end", job, cta, sw))
                if sw + 1 < J["iters"]:
                    yield from barrier(key)
        yield from barrier(key)  # end of the grid
        if J["staged"]:
            sh.log.append(("stage_out", job, cta, -1))


def plan(jobs, grid, ladder_want):
    """Tiers as the host builds them: the ladder grid, grid/2, ... 1; a job
    goes to the largest team at most its wanted size; jobs by tier."""
    ladder = []
    k = grid
    while k >= 1:
        ladder.append(k)
        k //= 2
    tier_of = []
    for j in jobs:
        w = max(1, min(ladder_want(j), grid))
        tier_of.append(next(i for i, v in enumerate(ladder) if v <= w))
    order = sorted(range(len(jobs)), key=lambda i: (tier_of[i], -jobs[i]["work"]))
    sorted_jobs = [jobs[i] for i in order]
    tiers = []
    for pos, i in enumerate(order):
        if not tiers or tiers[-1]["team"] != ladder[tier_of[i]]:
            tiers.append({"team": ladder[tier_of[i]], "first": pos, "njobs": 0})
        tiers[-1]["njobs"] += 1
    return tiers, sorted_jobs


def run(jobs, grid, want, seed, plant=False, skip_empty=False, max_steps=300_000):
    tiers, jobs = plan(jobs, grid, want)
    sh = Shared(len(tiers), grid)
    progs = {c: cta_program(c, grid, tiers, jobs, sh, plant, skip_empty) for c in range(grid)}
    rng = random.Random(seed)
    live = list(progs)
    steps = 0
    while live:
        c = rng.choice(live)
        try:
            next(progs[c])
        except StopIteration:
            live.remove(c)
        steps += 1
        assert steps < max_steps, "no progress: deadlock"
    return jobs, sh.log


def check(jobs, log):
    by_job = {}
    for ev, j, c, sw in log:
        by_job.setdefault(j, []).append((ev, c, sw))
    for j, J in enumerate(jobs):
        evs = by_job.get(j, [])
        if J["iters"] <= 0:
            assert not evs
            continue
        ctas = sorted({c for ev, c, _ in evs})
        assert ctas == list(range(ctas[0], ctas[-1] + 1)), "one contiguous team per grid"
        sweepers = sorted({c for ev, c, _ in evs if ev == "start"})
        if J["dims"] == 3:
            assert len(sweepers) == min(J["items"], len(ctas))
        for c in sweepers:
            assert [sw for ev, cc, sw in evs if cc == c and ev == "start"] == list(range(J["iters"]))
        # order: sweep s starts only after every sweeper ended sweep s-1
        ended = {}
        for ev, c, sw in evs:
            if ev == "start" and sw > 0:
                assert all(ended.get((cc, sw - 1)) for cc in sweepers), ("early sweep", j, c, sw)
            if ev == "end":
                ended[(c, sw)] = True
            if ev == "stage_out":
                assert all(ended.get((cc, J["iters"] - 1)) for cc in sweepers), "copy out before the last sweep"


def make_jobs(rng, n):
    jobs = []
    for _ in range(n):
        dims = rng.choice([2, 3])
        cells = int(rng.uniform(1e3, 5e6))
        jobs.append({"dims": dims, "iters": rng.choice([0, 1, 2, 3, 5]), "staged": rng.random() < 0.4,
                     "items": rng.randint(1, 40), "cells": cells, "work": cells})
    return jobs


@pytest.mark.parametrize("seed", range(12))
def test_protocol_every_grid_once_in_order_without_deadlock(seed):
    rng = random.Random(seed)
    grid = rng.choice([7, 12, 16, 19])
    jobs = make_jobs(rng, rng.randint(3, 14))
    cpc = rng.choice([1000, 100000, 10 ** 9])
    swept, log = run(jobs, grid, lambda j: j["cells"] // cpc, seed)
    check(swept, log)


def test_protocol_catches_idle_ctas_on_the_sweep_barrier():
    """The bug the team-size GPU tests found: CTAs without work items
    arriving at the 3-D sweep barrier let the others' producers pass it
    early.  Planted in the model, the order check fails."""
    jobs = [{"dims": 3, "iters": 6, "staged": False, "items": 3, "cells": 10 ** 6, "work": 1}]
    caught = 0
    for seed in range(20):
        swept, log = run(jobs, 8, lambda j: 8, seed, plant=True)
        try:
            check(swept, log)
        except AssertionError:
            caught += 1
    assert caught > 0


def test_protocol_catches_a_zero_sweep_grid_without_a_barrier():
    """The race this emulation found: a grid with no sweep used to end
    without a team barrier, so the leader could overwrite the mailbox before
    a teammate read it and the team split over two grids (a deadlock or a
    grid swept by part of its team).  Planted in the model, it is caught."""
    rng = random.Random(3)
    jobs = [{"dims": d, "iters": it, "staged": False, "items": 30, "cells": 10 ** 6, "work": w}
            for d, it, w in [(2, 3, 9), (3, 0, 8), (2, 0, 7), (3, 2, 6), (2, 4, 5)]]
    caught = 0
    for seed in range(20):
        try:
            swept, log = run(jobs, 12, lambda j: 12, seed, skip_empty=True)
            check(swept, log)
        except AssertionError:
            caught += 1
    assert caught > 0


def cta_program_bounded(cta, grid, tiers, jobs, sh, victim, die_after, limit):
    """The protocol with the kernel's failure handling: every wait gives up
    after `limit` steps (the kernel's bounded waits), sets the abort word and
    ends the CTA; a leader that sees the abort word hands its team the stop
    value instead of a grid.  CTA `victim` stops for good after `die_after`
    of its own steps, arriving nowhere again (a CTA whose wait gave up)."""
    steps = 0
    t, start, size, rel, cnt, job = -1, 0, grid, 0, 0, STOP

    def tick():
        nonlocal steps
        steps += 1
        return cta == victim and steps > die_after

    def barrier(key):
        nonlocal cnt
        sh.tbar[key] = sh.tbar.get(key, 0) + 1
        cnt += size
        spins = 0
        while sh.tbar[key] < cnt:
            spins += 1
            if spins > limit:
                sh.abort = True
                return False
            yield
        return True

    while True:
        while True:
            if t < 0 or job == STOP:
                t += 1
                if t >= len(tiers):
                    return
                start, size = split(start, size, tiers[t]["team"], cta)
                rel, cnt = cta - start, 0
            key = (t, start)
            if tick():
                return
            if rel == 0:
                if sh.abort:
                    sh.mail[key] = "stop"
                else:
                    sh.mail[key] = sh.queue[t]
                    sh.queue[t] += 1
                yield
            if not (yield from barrier(key)):
                return
            yield
            j = sh.mail[key]
            if j == "stop":
                return
            if j < tiers[t]["njobs"]:
                job = tiers[t]["first"] + j
                break
            job = STOP
        J = jobs[job]
        sh.log.append(("begin", job, cta, int(sh.abort)))
        for sw in range(max(1, J["iters"])):
            if tick():
                return
            yield
            if not (yield from barrier(key)):
                return


@pytest.mark.parametrize("seed", range(8))
def test_protocol_a_stopped_cta_ends_the_launch_without_a_hang(seed):
    """A CTA that stops mid-batch (its wait gave up): every other CTA ends
    within bounded waits -- its teammates time out and set the abort word,
    the other teams' leaders then hand out the stop value -- and no grid is
    begun by part of a team (CPU emulation; the kernel's waits are bounded
    by time)."""
    rng = random.Random(100 + seed)
    grid = rng.choice([8, 12, 16])
    jobs = make_jobs(rng, 12)
    tiers, jobs = plan(jobs, grid, lambda j: j["cells"] // 100000)
    sh = Shared(len(tiers), grid)
    sh.abort = False
    victim = rng.randrange(grid)
    progs = {c: cta_program_bounded(c, grid, tiers, jobs, sh, victim, rng.randint(1, 12), 400)
             for c in range(grid)}
    live = list(progs)
    steps = 0
    while live:
        c = rng.choice(live)
        try:
            next(progs[c])
        except StopIteration:
            live.remove(c)
        steps += 1
        assert steps < 2_000_000, "a CTA never ended"
    # every grid that began was handed out before its team's leader saw the
    # abort word, so each was begun by its whole team or by none of it
    begun = {}
    for ev, j, c, _ in sh.log:
        if ev == "begin":
            begun.setdefault(j, set()).add(c)
    for j, ctas in begun.items():
        assert sorted(ctas) == list(range(min(ctas), max(ctas) + 1)), ("part of a team", j)
