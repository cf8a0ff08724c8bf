"""GPU tests of the batched/served closure: every job's result is identical
alone and in the mix (integer work, so identical means bit-exact: per-label
counts and edge-set hash over job-local ids), including jobs admitted while
others are in flight and vertex ranges reused after release."""
import numpy as np
import pytest

import grg_gen as G
import serve

pytestmark = pytest.mark.gpu


def small_jobs(n=8, seed=17, vmin=400, vmax=2500):
    specs = G.batch_mix(seed=seed, jobs=n, vmin=vmin, vmax=vmax)
    return serve.make_jobs(specs, block=250)


def alone(oracle_mod, j):
    rules, labels = serve.GRAMMARS[j.grammar]
    rid = np.array([[labels.index(x) + 1 for x in r] + [0] * (3 - len(r)) for r in rules], dtype=np.int32)
    r = oracle_mod.closure(j.num_vars, rid, len(labels), 0, j.src, j.dst, j.lab)
    return [int(x) for x in r.label_counts()], r.set_hash


def test_batch_equals_alone_with_range_reuse(grg_mod, oracle_mod):
    jobs = small_jobs()
    # vertex space for about half the jobs at once: later jobs reuse released ranges
    max_vars = sum(j.num_vars for j in jobs) // 2 + max(j.num_vars for j in jobs)
    res = serve.serve(jobs, max_vars=max_vars, max_jobs=4, realtime=False)
    assert res["jobs"] == len(jobs)
    for j in jobs:
        counts, h = alone(oracle_mod, j)
        assert j.counts == counts, (j.job, j.kind)
        assert j.hash == h
    assert res["total_edges"] == sum(sum(alone(oracle_mod, j)[0]) for j in jobs)


def test_midflight_admission(grg_mod, oracle_mod):
    jobs = small_jobs(n=6, seed=23)
    ctx = grg_mod.Context(0)
    ctx.allocate_pool(0)
    b = grg_mod.Batch(ctx, sum(j.num_vars for j in jobs) + 10, 8, serve.GRAMMARS, 0)
    base = 0
    placed = {}

    def admit(k):
        nonlocal base
        j = jobs[k]
        b.admit(k, base, j.grammar, j.num_vars, j.src, j.dst, j.lab)
        placed[k] = base
        base += j.num_vars

    admit(0)
    admit(1)
    rec, _ = b.step(2)                       # two rounds of jobs 0 and 1
    # a job that has not reached its fixpoint cannot be released
    if rec[0] != 0:
        with pytest.raises(grg_mod.GrgError) as ei:
            b.release(0)
        assert ei.value.status == grg_mod.E_STATE
    for k in range(2, 6):
        admit(k)                             # admitted while 0 and 1 are in flight
        b.step(1)
    done = {}
    for _ in range(10000):
        rec, _ = b.step(1)
        for k in placed:
            if k not in done and rec[k] == 0:
                done[k] = b.result(k, jobs[k].grammar)
        if len(done) == len(placed):
            break
    for k, j in enumerate(jobs):
        counts, h = alone(oracle_mod, j)
        assert [int(x) for x in done[k][0]] == counts and done[k][1] == h, k
    ctx.close()


def test_plain_and_served_agree(grg_mod):
    jobs = small_jobs(n=6, seed=31)
    p = serve.plain(jobs)
    res = serve.serve(jobs, max_vars=sum(j.num_vars for j in jobs), max_jobs=8, realtime=False)
    assert [r[1] for r in p["results"]] == [j.counts for j in jobs]
    assert [r[2] for r in p["results"]] == [j.hash for j in jobs]
    assert res["total_edges"] == p["total_edges"]


def test_refused_admission_leaves_the_batch_usable(grg_mod, oracle_mod):
    # a job with an edge label outside the union grammar, or a vertex id beyond its
    # range, is refused; its slot and range are admitted again with valid edges
    jobs = small_jobs(n=2, seed=29)
    ctx = grg_mod.Context(0)
    ctx.allocate_pool(0)
    b = grg_mod.Batch(ctx, sum(j.num_vars for j in jobs) + 10, 4, serve.GRAMMARS, 0)
    j = jobs[0]
    lab = np.asarray(j.lab, np.int64).copy()
    lab[3] = 200 - b.offsets[j.grammar]          # label id 200 > every union label
    with pytest.raises(grg_mod.GrgError) as ei:
        b.admit(0, 0, j.grammar, j.num_vars, j.src, j.dst, lab)
    assert ei.value.status == grg_mod.E_LABEL
    dst = np.asarray(j.dst, np.uint32).copy()
    dst[4] = j.num_vars
    with pytest.raises(grg_mod.GrgError) as ei:
        b.admit(0, 0, j.grammar, j.num_vars, j.src, dst, j.lab)
    assert ei.value.status == grg_mod.E_RANGE
    base = 0
    for k, jj in enumerate(jobs):
        b.admit(k, base, jj.grammar, jj.num_vars, jj.src, jj.dst, jj.lab)
        base += jj.num_vars
    for _ in range(10000):
        rec, n = b.step(8)
        if n == 0 and not rec.any():
            break
    for k, jj in enumerate(jobs):
        counts, h = b.result(k, jj.grammar)
        assert ([int(x) for x in counts], h) == alone(oracle_mod, jj)
    ctx.close()


def test_admission_held_by_footprint_budget(grg_mod, oracle_mod):
    """With a budget of two jobs' projected footprints, arrived jobs wait for memory:
    the service admits at most what the budget holds (never more than one job beyond
    it, the one admitted into an empty batch), holds the rest back, and every result
    still equals the job closed alone."""
    jobs = small_jobs(n=8, seed=37)
    fps = sorted(serve.footprint_bytes(j) for j in jobs)
    budget = fps[-1] + fps[-2]
    res = serve.serve(jobs, max_vars=sum(j.num_vars for j in jobs), max_jobs=8, realtime=False,
                      budget_bytes=budget, rounds_per_step=1)
    assert res["held_by_budget"] > 0
    assert res["peak_projected_bytes"] <= budget
    for j in jobs:
        assert (j.counts, j.hash) == tuple(alone(oracle_mod, j))
