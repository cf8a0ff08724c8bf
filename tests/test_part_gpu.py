"""GPU tests of the out-of-core partitioned closure (grg_part_*) and of the
element-image calls it is built on. Integer work, so every comparison is
bit-exact: per-label counts and the edge-set hash equal the oracle's for any
number of partitions, for both schedules (stream: no derived second symbol;
pairs: supersteps over partition pairs), and when a small pool limit forces
partitions to split."""
import numpy as np
import pytest

import grg_gen as G

pytestmark = pytest.mark.gpu


def oracle_result(O, w, f):
    r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    return [int(x) for x in r.label_counts()], r.set_hash


def part_closure(grg, w, f, parts, pool_bytes=0):
    ctx = grg.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    if pool_bytes:
        ctx.set_pool_limit(pool_bytes)
    p = grg.Partitioned(ctx, w.num_vars, parts)
    p.load_edges(w.src, w.dst, w.lab)
    st = p.run(f)
    counts, h = p.label_counts()
    bounds = p.bounds()
    p.close()
    ctx.close()
    return [int(x) for x in counts], h, st, bounds


@pytest.mark.parametrize("parts", [1, 2, 3, 7])
def test_pointsto_pairs(grg_mod, oracle_mod, parts):
    w = G.pointsto(seed=5, num_vars=600, num_edges=1500)
    want = oracle_result(oracle_mod, w, 0)
    counts, h, st, bounds = part_closure(grg_mod, w, 0, parts)
    assert (counts, h) == want
    assert st["schedule"] == "pairs"
    assert st["total_edges"] == sum(want[0])
    assert st["num_parts"] == parts and len(bounds) == parts + 1
    assert bounds[0] == 0 and bounds[-1] == w.num_vars and np.all(np.diff(bounds) > 0)
    if parts > 1:
        # the last superstep runs nothing; pairs without news are skipped
        assert st["supersteps"] >= 2 and st["skipped"] > 0


def test_alias_pairs(grg_mod, oracle_mod):
    w = G.alias(seed=9, num_vars=3000, num_base_edges=6000, block=500)
    want = oracle_result(oracle_mod, w, 0)
    counts, h, st, _ = part_closure(grg_mod, w, 0, 4)
    assert (counts, h) == want and st["schedule"] == "pairs"


@pytest.mark.parametrize("f", [0, 1])
def test_dataflow_stream(grg_mod, oracle_mod, f):
    w = G.dataflow_blocks(seed=11, num_blocks=6, block=500, num_edges=9000)
    want = oracle_result(oracle_mod, w, f)
    counts, h, st, _ = part_closure(grg_mod, w, f, 4)
    assert (counts, h) == want
    assert st["schedule"] == "stream" and st["runs"] == 4 and st["supersteps"] == 0
    # each partition's input after the first was assembled and copied while the one before computed
    assert st["prefetched"] == 3 and st["prefetch_hits"] == 3


@pytest.mark.parametrize("seed", range(8))
def test_random_grammars_partitioned(grg_mod, oracle_mod, seed):
    w = G.random_grammar_graph(300 + seed, num_vars=150 + 31 * seed, num_edges=300 + 40 * seed,
                               num_labels=3 + seed % 4, num_rules=3 + seed % 5)
    for f in (0, 1):
        try:
            want = oracle_result(oracle_mod, w, f)
        except oracle_mod.OracleError as e:
            assert e.code == oracle_mod.ORC_E_FILTER
            with pytest.raises(grg_mod.GrgError) as ei:
                part_closure(grg_mod, w, f, 3)
            assert ei.value.status == grg_mod.E_FILTER
            continue
        counts, h, _, _ = part_closure(grg_mod, w, f, 3)
        assert (counts, h) == want, (seed, f)


def in_core_pool_bytes(grg, w, f):
    ctx, st = grg.run_closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    ctx.close()
    return st["pool_elems_used"] * 69          # element, delta bitmap, dirty bit, stamp


def test_splits_under_pool_limit(grg_mod, oracle_mod):
    # a third of what the in-core closure used: partitions split until every run fits
    w = G.pointsto(seed=7, num_vars=1200, num_edges=3000)
    want = oracle_result(oracle_mod, w, 0)
    counts, h, st, bounds = part_closure(grg_mod, w, 0, 2, pool_bytes=in_core_pool_bytes(grg_mod, w, 0) // 3)
    assert (counts, h) == want
    assert st["splits"] > 0 and st["num_parts"] > 2 and len(bounds) == st["num_parts"] + 1
    w2 = G.dataflow_blocks(seed=12, num_blocks=8, block=500, num_edges=12000)
    want2 = oracle_result(oracle_mod, w2, 1)
    counts2, h2, st2, _ = part_closure(grg_mod, w2, 1, 1, pool_bytes=in_core_pool_bytes(grg_mod, w2, 1) // 3)
    assert (counts2, h2) == want2
    assert st2["splits"] > 0 and st2["schedule"] == "stream"


def test_element_image_round_trip(grg_mod, oracle_mod):
    w = G.pointsto(seed=13, num_vars=500, num_edges=1200)
    want = oracle_result(oracle_mod, w, 0)
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    ctx.closure(0)
    recs, stamps = ctx.export_elements()
    assert recs.shape[1] == 8 and len(stamps) == len(recs)
    # rows are where they were exported from, keys name labels 1..L
    assert np.all(recs[:, 7] < w.num_vars)
    assert np.all((recs[:, 6] >> 25) >= 1) and np.all((recs[:, 6] >> 25) <= w.num_labels)
    # halves of the vertex range partition the image
    a, _ = ctx.export_elements(0, 250)
    b, _ = ctx.export_elements(250, w.num_vars)
    assert len(a) + len(b) == len(recs)
    ca, ha = ctx.range_counts(0, 250)
    cb, hb = ctx.range_counts(250, w.num_vars)
    assert [int(x) for x in ca + cb] == want[0] and (ha + hb) % 2**64 == want[1]
    # reloading the closed image (nothing marked) changes nothing
    ctx2 = grg_mod.Context(0)
    ctx2.transfer_rules(w.rule_ids(), w.num_labels)
    ctx2.load_elements(w.num_vars, recs, np.ones(len(recs), np.uint32), mark_after=1)
    st = ctx2.closure_ex(0, 2)
    assert st["rounds"] == 0
    assert ([int(x) for x in ctx2.label_counts()], ctx2.set_hash()) == want
    # reloading it with every element marked reaches the same fixpoint; nothing is restamped
    ctx2.load_elements(w.num_vars, recs, np.ones(len(recs), np.uint32), mark_after=0)
    st = ctx2.closure_ex(0, 2)
    assert st["rounds"] == 1
    _, st2 = ctx2.export_elements()
    assert np.all(st2 == 1)
    assert ([int(x) for x in ctx2.label_counts()], ctx2.set_hash()) == want
    # repeated and out-of-range records are refused
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx2.load_elements(w.num_vars, np.concatenate([recs, recs[:1]]), np.ones(len(recs) + 1, np.uint32))
    assert ei.value.status == grg_mod.E_ARG
    bad = recs[:1].copy()
    bad[0, 7] = w.num_vars
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx2.load_elements(w.num_vars, bad, np.ones(1, np.uint32))
    assert ei.value.status == grg_mod.E_ARG
    ctx.close()
    ctx2.close()


def test_range_reach_matches_edges(grg_mod):
    # reach of a vertex range = the partitions its B-label edges end in (a superset at most)
    w = G.pointsto(seed=17, num_vars=700, num_edges=1600)
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    bounds = np.array([0, 100, 250, 251, 400, 700], np.uint32)
    ids = w.rule_ids()
    bmask = 0
    for r in ids:
        if r[1] and r[2]:
            bmask |= 1 << (int(r[1]) - 1)
    for lo, hi in [(0, 100), (100, 400), (250, 251), (0, 700)]:
        got = ctx.range_reach(lo, hi, bmask, bounds)
        sel = (w.src >= lo) & (w.src < hi) & (((bmask >> (w.lab.astype(np.int64) - 1)) & 1) == 1)
        want = np.zeros(len(bounds) - 1, bool)
        for d in w.dst[sel]:
            want[np.searchsorted(bounds, d, side="right") - 1] = True
        assert np.all(got[want] == 1), (lo, hi)          # never one too few
    ctx.close()


def test_block_graph_needs_no_cross_pairs(grg_mod, oracle_mod):
    # block-confined alias graph, partitions on block boundaries: self-runs only, no pair runs
    w = G.alias(seed=19, num_vars=4000, num_base_edges=8000, block=500)
    want = oracle_result(oracle_mod, w, 0)
    counts, h, st, bounds = part_closure(grg_mod, w, 0, 8)
    assert (counts, h) == want
    assert st["runs"] == 8 and st["supersteps"] == 2
