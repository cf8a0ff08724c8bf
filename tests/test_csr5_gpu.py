"""GPU tests of the compressed edge stream (grg_export_csr5 / grg_load_csr5)
and of the refusal of invalid input edges by every load path. Byte work, so
every comparison is bit-exact against the oracle's writer."""
import numpy as np
import pytest

import grg_gen as G
from test_csr5 import pack_csr5, unpack_csr5

pytestmark = pytest.mark.gpu

WORKLOADS = [
    ("pointsto", lambda: G.pointsto(seed=41, num_vars=900, num_edges=2500), 0),
    ("dataflow", lambda: G.dataflow_blocks(seed=42, num_blocks=4, block=500, num_edges=6000), 1),
    ("alias", lambda: G.alias(seed=43, num_vars=3000, num_base_edges=7000, block=500), 0),
]


def closed_context(grg, w, f):
    ctx = grg.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    ctx.closure(f)
    return ctx


@pytest.mark.parametrize("name,make,f", WORKLOADS, ids=[x[0] for x in WORKLOADS])
def test_export_matches_oracle_stream(grg_mod, oracle_mod, name, make, f):
    w = make()
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    ctx = closed_context(grg_mod, w, f)
    V = w.num_vars
    for lo, hi in [(0, V), (0, 1), (V // 4, V // 2), (V - 1, V), (7, 7)]:
        got, deg = ctx.export_csr5(lo, hi)
        want, wdeg = r.csr5(lo, hi)
        assert len(got) == len(want), (lo, hi)
        assert np.array_equal(got, want), (lo, hi)
        assert np.array_equal(deg, wdeg), (lo, hi)
    ctx.close()


def test_random_grammars_export(grg_mod, oracle_mod):
    for seed in range(6):
        w = G.random_grammar_graph(500 + seed, num_vars=200 + 37 * seed, num_edges=500 + 60 * seed,
                                   num_labels=3 + seed % 4, num_rules=3 + seed % 5)
        r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
        ctx = closed_context(grg_mod, w, 0)
        got, deg = ctx.export_csr5()
        want, wdeg = r.csr5()
        assert np.array_equal(got, want) and np.array_equal(deg, wdeg), seed
        ctx.close()


def test_load_of_input_stream_equals_load_of_edges(grg_mod, oracle_mod):
    # a grammar without epsilon rules: the stream load applies none (a spilled image holds its own)
    w = G.alias(seed=44, num_vars=1600, num_base_edges=4000, block=400)
    want = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    stream, deg = pack_csr5(w.src, w.dst, w.lab, 0, w.num_vars)
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_csr5(w.num_vars, stream, deg)
    ctx.closure(0)
    assert [int(x) for x in ctx.label_counts()] == [int(x) for x in want.label_counts()]
    assert ctx.set_hash() == want.set_hash
    got, gdeg = ctx.export_csr5()
    ws, wd = want.csr5()
    assert np.array_equal(got, ws) and np.array_equal(gdeg, wd)
    ctx.close()


def test_closed_stream_reloads_to_the_same_fixpoint(grg_mod, oracle_mod):
    # the points-to grammar has epsilon rules: the closed stream carries their edges
    w = G.pointsto(seed=45, num_vars=900, num_edges=2400)
    want = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    ctx = closed_context(grg_mod, w, 0)
    stream, deg = ctx.export_csr5()
    ctx2 = grg_mod.Context(0)
    ctx2.transfer_rules(w.rule_ids(), w.num_labels)
    ctx2.load_csr5(w.num_vars, stream, deg)
    ctx2.closure(0)
    assert [int(x) for x in ctx2.label_counts()] == [int(x) for x in want.label_counts()]
    assert ctx2.set_hash() == want.set_hash
    ctx.close()
    ctx2.close()


def test_partial_range_stream(grg_mod):
    # the stream of rows [a, b) holds exactly the input edges leaving those rows
    w = G.alias(seed=46, num_vars=1200, num_base_edges=3600, block=400)
    a, b = 300, 700
    stream, deg = pack_csr5(w.src, w.dst, w.lab, a, b)
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_csr5(w.num_vars, stream, deg, v_begin=a)
    got, gdeg = ctx.export_csr5(0, w.num_vars)
    assert np.array_equal(gdeg[:a], np.zeros(a, np.uint32)) and np.all(gdeg[b:] == 0)
    assert np.array_equal(got, stream) and np.array_equal(gdeg[a:b], deg)
    ctx.close()


def test_invalid_streams_are_refused(grg_mod):
    w = G.pointsto(seed=47, num_vars=400, num_edges=1000)
    stream, deg = pack_csr5(w.src, w.dst, w.lab, 0, w.num_vars)
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    # lengths that do not add up
    bad = deg.copy()
    bad[3] += 1
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx.load_csr5(w.num_vars, stream, bad)
    assert ei.value.status == grg_mod.E_ARG
    # a label outside 1..L
    s2 = stream.copy().reshape(-1, 5)
    s2[10, 4] = w.num_labels + 1
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx.load_csr5(w.num_vars, s2.reshape(-1), deg)
    assert ei.value.status == grg_mod.E_LABEL
    s2[10, 4] = 0
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx.load_csr5(w.num_vars, s2.reshape(-1), deg)
    assert ei.value.status == grg_mod.E_LABEL
    # a destination beyond the graph
    s3 = stream.copy().reshape(-1, 5)
    s3[20, :4] = np.frombuffer(np.uint32(w.num_vars).tobytes(), np.uint8)
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx.load_csr5(w.num_vars, s3.reshape(-1), deg)
    assert ei.value.status == grg_mod.E_RANGE
    # a row whose edges are out of order splits a record in two: refused as a repeat
    def rec(dst, lab):
        return list(np.frombuffer(np.uint32(dst).tobytes(), np.uint8)) + [lab]
    s4 = np.array(rec(1, 1) + rec(3, 2) + rec(2, 1), np.uint8)
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx.load_csr5(w.num_vars, s4, np.array([3], np.uint32))
    assert ei.value.status == grg_mod.E_ARG
    # the context still loads and closes a valid stream
    ctx.load_csr5(w.num_vars, stream, deg)
    ctx.closure(0)
    assert sum(int(x) for x in ctx.label_counts()) >= len(w.src)
    ctx.close()


def test_invalid_edges_are_refused_by_every_load_path(grg_mod, oracle_mod):
    w = G.pointsto(seed=48, num_vars=300, num_edges=800)
    want = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    cases = []
    lab = w.lab.copy(); lab[5] = w.num_labels + 1
    cases.append((w.src, w.dst, lab, grg_mod.E_LABEL))
    lab = w.lab.copy(); lab[6] = 0
    cases.append((w.src, w.dst, lab, grg_mod.E_LABEL))
    src = w.src.copy(); src[7] = w.num_vars
    cases.append((src, w.dst, w.lab, grg_mod.E_RANGE))
    dst = w.dst.copy(); dst[8] = 0xFFFFFFFF
    cases.append((w.src, dst, w.lab, grg_mod.E_RANGE))
    ctx = grg_mod.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    for s, d, l, code in cases:
        with pytest.raises(grg_mod.GrgError) as ei:
            ctx.load_edges(w.num_vars, s, d, l)
        assert ei.value.status == code
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    ctx.closure(0)
    assert ctx.set_hash() == want.set_hash
    ctx.close()


def test_export_in_pieces_under_a_small_budget(grg_mod, oracle_mod, monkeypatch):
    # a device budget of a few tens of KB splits the range into many row pieces; their
    # streams and row lengths concatenate to the oracle's
    w = G.alias(seed=49, num_vars=3000, num_base_edges=7000, block=500)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    ctx = closed_context(grg_mod, w, 0)
    monkeypatch.setenv("GRG_CSR5_BUDGET", "40000")
    for lo, hi in [(0, w.num_vars), (123, 2500)]:
        got, deg = ctx.export_csr5(lo, hi)
        want, wdeg = r.csr5(lo, hi)
        assert np.array_equal(got, want) and np.array_equal(deg, wdeg), (lo, hi)
    ctx.close()


def test_load_in_pieces_under_a_small_budget(grg_mod, oracle_mod, monkeypatch):
    # a host stream larger than the budget goes to the device in row pieces whose records
    # are joined before the load; the closure is the oracle's
    w = G.pointsto(seed=50, num_vars=900, num_edges=2400)
    want = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    ctx = closed_context(grg_mod, w, 0)
    stream, deg = ctx.export_csr5()
    ctx.close()
    monkeypatch.setenv("GRG_CSR5_BUDGET", "20000")
    ctx2 = grg_mod.Context(0)
    ctx2.transfer_rules(w.rule_ids(), w.num_labels)
    ctx2.load_csr5(w.num_vars, stream, deg)
    got, gdeg = ctx2.export_csr5()
    assert np.array_equal(got, stream) and np.array_equal(gdeg, deg)
    ctx2.closure(0)
    assert [int(x) for x in ctx2.label_counts()] == [int(x) for x in want.label_counts()]
    assert ctx2.set_hash() == want.set_hash
    # a bad label in a late piece is still refused
    s2 = stream.copy().reshape(-1, 5)
    s2[-3, 4] = w.num_labels + 1
    with pytest.raises(grg_mod.GrgError) as ei:
        ctx2.load_csr5(w.num_vars, s2.reshape(-1), deg)
    assert ei.value.status == grg_mod.E_LABEL
    ctx2.close()
