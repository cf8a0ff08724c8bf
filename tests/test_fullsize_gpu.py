"""GPU parity at the measured sizes: the alias closures of 1M and 8M vertices
(in core, and the 8M one also over 64 out-of-core partitions) and a sample of
the 512-job mix closed in one batch, each against the CPU oracle's figures in
tests/golden/golden.json (per-label counts and the order-independent edge-set
hash; integer work, so equal means bit-exact). The oracle takes about 40 s for
the 1M-vertex closure and several minutes for the 8M-vertex one, so its
results are recorded by tests/golden/make_golden.py rather than recomputed."""
import json
import os

import pytest

import grg_gen as G

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
C4_ARGS = dict(seed=0x5EED0004, num_vars=8_000_000, num_base_edges=40_000_000, block=1000)


def _closed(grg, w):
    ctx = grg.Context(0)
    ctx.allocate_pool(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    st = ctx.closure(w.filter_flag)
    return ctx, st


def test_alias_1m_full_size(grg_mod):
    """1M vertices, 4M base + 4M inverse edges: 2,375,361,416 closure edges."""
    g = GOLD["alias_c3"]
    w = G.alias()
    assert w.num_edges == g["num_edges"]
    ctx, st = _closed(grg_mod, w)
    assert st["total_edges"] == g["total"] == 2_375_361_416
    assert st["rounds"] == g["rounds"]
    assert dict(zip(w.labels, ctx.label_counts().tolist())) == g["labels"]
    assert ctx.set_hash() == g["hash"]
    ctx.close()


@pytest.mark.skipif("alias_c4" not in GOLD, reason="8M-vertex oracle figures not recorded")
def test_alias_8m_in_core_and_partitioned(grg_mod):
    """8M vertices, 40M base + 40M inverse edges, in core and over 64
    vertex-range partitions through host memory."""
    g = GOLD["alias_c4"]
    w = G.alias(**C4_ARGS)
    assert w.num_edges == g["num_edges"]
    ctx, st = _closed(grg_mod, w)
    assert st["total_edges"] == g["total"]
    assert dict(zip(w.labels, ctx.label_counts().tolist())) == g["labels"]
    assert ctx.set_hash() == g["hash"]
    ctx.close()
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    part = grg_mod.Partitioned(ctx, w.num_vars, 64)
    part.load_edges(w.src, w.dst, w.lab)
    pst = part.run(w.filter_flag)
    counts, h = part.label_counts()
    assert pst["total_edges"] == g["total"]
    assert dict(zip(w.labels, [int(x) for x in counts])) == g["labels"]
    assert h == g["hash"]
    part.close()
    ctx.close()


def test_batch_mix_sample(grg_mod):
    """Every 16th job of the 512-job mix (both grammars, 1k-200k vertices),
    closed together in one batch: each job's counts and hash equal the oracle's
    for the job closed alone."""
    import serve
    g = GOLD["batch_mix_sample"]
    specs = G.batch_mix()[::g["stride"]]
    jobs = serve.make_jobs(specs)
    assert [j.job for j in jobs] == [x["job"] for x in g["jobs"]]
    res = serve.serve(jobs, max_vars=sum(j.num_vars for j in jobs) + 1, max_jobs=len(jobs), realtime=False)
    assert res["jobs"] == len(jobs)
    for j, want in zip(jobs, g["jobs"]):
        assert j.num_vars == want["num_vars"] and len(j.src) == want["num_edges"]
        assert j.counts == want["labels"], (j.job, j.kind)
        assert j.hash == want["hash"], (j.job, j.kind)


def test_alias_8m_cross_partition_pairs(grg_mod, oracle_mod):
    """The 8M-vertex alias graph with 2% of its edges calling the partner block
    125 blocks away -- across the boundary of the 64 partitions of 125 blocks --
    so the pairs schedule must run cross pairs. In-core and out-of-core closures
    agree; 16 sampled two-block components are closed by the oracle alone and
    match the GPU's range counts and hashes over their rows."""
    import numpy as np
    w = G.alias(seed=0x5EED0006, num_vars=8_000_000, num_base_edges=40_000_000, block=1000, partner=125)
    ctx = grg_mod.Context(0)
    ctx.allocate_pool(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    st = ctx.closure(0)
    whole = ([int(x) for x in ctx.label_counts()], ctx.set_hash())
    # components {b, b + 125} for b // 125 even: sample 16 of them
    comps = [(b, b + 125) for b in range(0, 8000, 500)][:16]
    got_counts = np.zeros(w.num_labels, np.uint64)
    got_hash = 0
    for b0, b1 in comps:
        for b in (b0, b1):
            c, h = ctx.range_counts(b * 1000, (b + 1) * 1000)
            got_counts += c
            got_hash = (got_hash + h) & (2**64 - 1)
    ctx.close()
    rows = np.zeros(w.num_vars, bool)
    for b0, b1 in comps:
        rows[b0 * 1000:(b0 + 1) * 1000] = True
        rows[b1 * 1000:(b1 + 1) * 1000] = True
    sel = rows[w.src]
    assert rows[w.dst[sel]].all()                    # the sampled components are closed
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src[sel], w.dst[sel], w.lab[sel])
    assert got_counts.tolist() == r.label_counts().tolist() and got_hash == r.set_hash
    # out of core over 64 partitions: cross pairs run, the result equals the in-core one
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    part = grg_mod.Partitioned(ctx, w.num_vars, 64)
    part.load_edges(w.src, w.dst, w.lab)
    pst = part.run(0)
    counts, h = part.label_counts()
    assert ([int(x) for x in counts], h) == whole
    assert pst["total_edges"] == st["total_edges"]
    # the 32 partner pairs (p, p + 1), p even, run as cross pairs (a run closes both its
    # partitions' own rows, so no self-run is left); the plain C4 graph runs 64 self-runs
    assert pst["schedule"] == "pairs" and 32 <= pst["runs"] < 64 and pst["supersteps"] >= 2
    part.close()
    ctx.close()
