"""CPU tests of the oracle: pinned against the independent pure-Python fixpoint
and the figures recorded in tests/golden/golden.json."""
import json
import os

import numpy as np
import pytest

import grg_gen as G
import naive_cfl
from conftest import REFERENCE_SAMPLE

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _oracle_set(O, w, filter_flag=None):
    f = w.filter_flag if filter_flag is None else filter_flag
    r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    s, d, l = r.edges()
    return r, set(zip(s.tolist(), d.tolist(), l.tolist()))


def test_reference_sample_figure(oracle_mod):
    O = oracle_mod
    g = O.parse_grammar(os.path.join(REFERENCE_SAMPLE, "rules_pointsto.txt"))
    assert g.num_labels == 13 and len(g.rules) == 12
    # labels numbered by first appearance (src/main.cpp:84-88)
    assert g.labels[:5] == ["M", "DV", "d", "-d", "V"]
    nv, s, d, l = O.parse_graph(os.path.join(REFERENCE_SAMPLE, "programGraph_sample_pointsto.txt"), g)
    assert nv == 530 and len(s) == 2000
    r = O.closure(nv, g.rules, g.num_labels, 0, s, d, l)
    assert r.total == 3246
    counts = dict(zip(g.labels, r.label_counts().tolist()))
    assert counts == {"M": 0, "DV": 0, "d": 352, "-d": 0, "V": 591, "MAM": 530, "AMs": 591, "MAs": 530,
                      "Mq": 530, "MA": 0, "-a": 0, "AM": 61, "a": 61}
    assert r.set_hash == GOLD["reference_sample"]["hash"]
    ref = naive_cfl.closure(nv, g.rules, zip(s.tolist(), d.tolist(), l.tolist()), 0)
    es, ed, el = r.edges()
    assert set(zip(es.tolist(), ed.tolist(), el.tolist())) == ref


@pytest.mark.parametrize("seed", range(40))
def test_oracle_matches_naive_random(oracle_mod, seed):
    O = oracle_mod
    w = G.random_grammar_graph(seed, num_vars=int(30 + seed * 7), num_edges=60 + seed * 5,
                               num_labels=3 + seed % 4, num_rules=3 + seed % 6)
    for f in (0, 1):
        try:
            ref = naive_cfl.closure(w.num_vars, w.rule_ids(), zip(w.src.tolist(), w.dst.tolist(), w.lab.tolist()), f)
        except ValueError:
            with pytest.raises(O.OracleError) as ei:
                _oracle_set(O, w, f)
            assert ei.value.code == O.ORC_E_FILTER
            continue
        _, got = _oracle_set(O, w, f)
        assert got == ref


def test_oracle_matches_naive_pointsto_small(oracle_mod):
    w = G.pointsto(seed=7, num_vars=300, num_edges=600)
    ref = naive_cfl.closure(w.num_vars, w.rule_ids(), zip(w.src.tolist(), w.dst.tolist(), w.lab.tolist()), 0)
    _, got = _oracle_set(oracle_mod, w)
    assert got == ref


def test_filter1_refused_when_schedule_dependent(oracle_mod):
    O = oracle_mod
    # A ::= A A: second symbol derivable -> filter 1 is schedule-dependent
    with pytest.raises(O.OracleError) as ei:
        O.closure(4, [[1, 1, 1]], 1, 1, np.array([0, 1], np.uint32), np.array([1, 2], np.uint32),
                  np.array([1, 1], np.uint8))
    assert ei.value.code == O.ORC_E_FILTER


def test_filter0_eonly_equals_filter1_seeded(oracle_mod):
    """closure(filter 0, e only) == closure(filter 1, e + N seeds) for N ::= N e | e."""
    O = oracle_mod
    w1 = G.dataflow_blocks(seed=11, num_blocks=12, num_edges=36_000, seed_n=True)
    w0 = G.dataflow_blocks(seed=11, num_blocks=12, num_edges=36_000, seed_n=False)
    r1 = O.closure(w1.num_vars, w1.rule_ids(), w1.num_labels, 1, w1.src, w1.dst, w1.lab)
    r0 = O.closure(w0.num_vars, w0.rule_ids(), w0.num_labels, 0, w0.src, w0.dst, w0.lab)
    assert r0.total == r1.total and r0.set_hash == r1.set_hash


def test_golden_small_workloads(oracle_mod):
    O = oracle_mod
    for name, w in (("dataflow_small", G.dataflow_small()),
                    ("dataflow_blocks_b100", G.dataflow_blocks(num_blocks=100, num_edges=300_000)),
                    ("alias_20k", G.alias(num_vars=20_000, num_base_edges=80_000))):
        g = GOLD[name]
        assert w.num_edges == g["num_edges"]
        r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, w.filter_flag, w.src, w.dst, w.lab)
        assert r.total == g["total"] and r.set_hash == g["hash"] and r.rounds == g["rounds"]


def test_row_mask_sample_equals_restriction(oracle_mod):
    """Filter-1 rows are independent: closing a subset of source rows gives
    exactly the full closure restricted to them (the CPU-baseline sample)."""
    O = oracle_mod
    w = G.dataflow_blocks(seed=5, num_blocks=20, num_edges=60_000)
    full = O.closure(w.num_vars, w.rule_ids(), w.num_labels, 1, w.src, w.dst, w.lab)
    mask = ((np.arange(w.num_vars) // 1000) % 4 == 1).astype(np.uint8)
    part = O.closure(w.num_vars, w.rule_ids(), w.num_labels, 1, w.src, w.dst, w.lab, row_mask=mask)
    fs, fd, fl = full.edges()
    keep = mask[fs] == 1
    ps, pd, pl = part.edges()
    assert np.array_equal(fs[keep], ps) and np.array_equal(fd[keep], pd) and np.array_equal(fl[keep], pl)


def test_epsilon_and_unary_only(oracle_mod):
    O = oracle_mod
    # A ::= eps ; B ::= A  over 5 vertices, no edges
    r = O.closure(5, [[1, 0, 0], [2, 1, 0]], 2, 0, np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                  np.zeros(0, np.uint8))
    assert r.total == 10
    assert r.label_counts().tolist() == [5, 5]
    # filter 1 keeps epsilon, drops unary
    r = O.closure(5, [[1, 0, 0], [2, 1, 0]], 2, 1, np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                  np.zeros(0, np.uint8))
    assert r.label_counts().tolist() == [5, 0]
