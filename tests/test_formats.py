"""CPU tests of the text formats, the generators and the C ABI surface."""
import ctypes
import os
import re

import numpy as np
import pytest

import grg_gen as G
from conftest import REFERENCE_SAMPLE, ROOT


def test_library_exports_every_declared_symbol(grg_mod):
    lib = grg_mod.load_library()
    header = open(os.path.join(ROOT, "include", "grg.h")).read()
    declared = set(re.findall(r"\b(grg_[a-z0-9_]+)\s*\(", header))
    assert declared == set(grg_mod.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_create_without_gpu_reports_nodev(grg_mod):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    lib = grg_mod.load_library()
    h = ctypes.c_void_p()
    assert lib.grg_create(ctypes.byref(h), 0) == grg_mod.E_NODEV
    assert "device" in grg_mod.error_string(grg_mod.E_NODEV)


def _write(tmp_path, w):
    gp = os.path.join(tmp_path, "rules.txt")
    fp = os.path.join(tmp_path, "graph.txt")
    G.write_grammar(gp, w.rules)
    G.write_graph(fp, w)
    return gp, fp


@pytest.mark.parametrize("make", [lambda: G.pointsto(num_vars=400, num_edges=1200),
                                  lambda: G.dataflow_small(num_vars=1000, num_edges=3000),
                                  lambda: G.alias(num_vars=3000, num_base_edges=9000)])
def test_parsers_match_oracle_and_generator(tmp_path, grg_mod, oracle_mod, make):
    w = make()
    gp, fp = _write(str(tmp_path), w)
    g = grg_mod.parse_grammar(gp)
    go = oracle_mod.parse_grammar(gp)
    assert g.labels == go.labels == w.labels
    assert np.array_equal(g.rules, go.rules) and np.array_equal(g.rules, w.rule_ids())
    nv, s, d, l = grg_mod.parse_graph(fp, g)
    nvo, so, do, lo = oracle_mod.parse_graph(fp, go)
    assert nv == nvo == w.num_vars
    assert np.array_equal(s, so) and np.array_equal(d, do) and np.array_equal(l, lo)
    order = np.lexsort((w.lab, w.dst, w.src))
    assert np.array_equal(s, w.src[order]) and np.array_equal(d, w.dst[order]) and np.array_equal(l, w.lab[order])


def test_parsers_on_reference_sample(grg_mod, oracle_mod):
    gp = os.path.join(REFERENCE_SAMPLE, "rules_pointsto.txt")
    fp = os.path.join(REFERENCE_SAMPLE, "programGraph_sample_pointsto.txt")
    g, go = grg_mod.parse_grammar(gp), oracle_mod.parse_grammar(gp)
    assert g.labels == go.labels and np.array_equal(g.rules, go.rules)
    # epsilon rules (Mq, MAs, AMs) have both RHS 0; Mq ::= M is unary
    eps = [g.labels[r[0] - 1] for r in g.rules if r[1] == 0]
    assert eps == ["Mq", "MAs", "AMs"]
    a, b = grg_mod.parse_graph(fp, g), oracle_mod.parse_graph(fp, go)
    assert a[0] == b[0] == 530
    for x, y in zip(a[1:], b[1:]):
        assert np.array_equal(x, y)


def test_parse_errors(tmp_path, grg_mod):
    gp = os.path.join(str(tmp_path), "g.txt")
    with open(gp, "w") as f:
        f.write("# c\n2\nN\tN\te\nN\te\n")
    g = grg_mod.parse_grammar(gp)
    assert g.labels == ["N", "e"] and g.rules.tolist() == [[1, 1, 2], [1, 2, 0]]
    fp = os.path.join(str(tmp_path), "x.txt")
    with open(fp, "w") as f:
        f.write("2\t3\n0\t1\te\n1\t2\tq\n")
    with pytest.raises(grg_mod.GrgError) as ei:
        grg_mod.parse_graph(fp, g)
    assert ei.value.status == grg_mod.E_LABEL
    with open(fp, "w") as f:
        f.write("2\t3\n0\t1\te\n1\t3\te\n")
    with pytest.raises(grg_mod.GrgError) as ei:
        grg_mod.parse_graph(fp, g)
    assert ei.value.status == grg_mod.E_RANGE
    # CRLF line endings and comment lines between edges
    with open(fp, "w") as f:
        f.write("# hdr\r\n2\t3\r\n0\t1\te\r\n# mid\r\n1\t2\tN\r\n")
    nv, s, d, l = grg_mod.parse_graph(fp, g)
    assert nv == 3 and s.tolist() == [0, 1] and d.tolist() == [1, 2] and l.tolist() == [2, 1]


def test_generators_shapes():
    w = G.dataflow_small()
    assert w.num_vars == 10_000 and w.num_edges == 30_000
    assert np.all(np.diff(w.src.astype(np.int64)) >= 0)
    key = w.src.astype(np.int64) * 10_000 + w.dst
    assert len(np.unique(key)) == w.num_edges
    deg = np.bincount(w.src, minlength=w.num_vars)
    assert deg.max() <= 64
    wb = G.dataflow_blocks(num_blocks=50, num_edges=150_000)
    n_id, e_id = wb.labels.index("N") + 1, wb.labels.index("e") + 1
    assert (wb.lab == n_id).sum() == (wb.lab == e_id).sum()
    e = wb.lab == e_id
    s, d = wb.src[e].astype(np.int64), wb.dst[e].astype(np.int64)
    pos_s, pos_d = s % 1000, d % 1000
    cross = (s // 1000) != (d // 1000)
    assert np.all(pos_s[cross] >= 990) and np.all(pos_d[cross] < 10)
    assert np.all(pos_d[~cross] < 990)
    assert abs(cross.mean() - 0.15) < 0.02
    wa = G.alias(num_vars=5000, num_base_edges=20_000)
    ids = {n: wa.labels.index(n) + 1 for n in wa.labels}
    assert wa.labels == ["V", "a", "a_bar", "M", "d_bar", "T", "d"]
    assert (wa.lab == ids["a"]).sum() == (wa.lab == ids["a_bar"]).sum()
    assert np.all(wa.src // 1000 == wa.dst // 1000)


def test_batch_mix_shape():
    jobs = G.batch_mix()
    assert len(jobs) == 512
    v = np.array([j["num_vars"] for j in jobs])
    assert v.min() >= 1000 and v.max() <= 200_000
    t = np.array([j["arrival_s"] for j in jobs])
    assert np.all(np.diff(t) > 0)
