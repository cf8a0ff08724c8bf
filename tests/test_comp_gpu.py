"""Tests of the `comp` command line (the reference's src/main.cpp:860-921
entry point): its stdout lines, the in-core and partitioned paths, the
compressed edge stream it writes, and resuming from a checkpoint file."""
import os
import re
import subprocess

import numpy as np
import pytest

import grg_gen as G


def comp_path(grg):
    return grg.COMP_PATH


def write_inputs(tmp, w):
    gp, fp = os.path.join(tmp, "rules.txt"), os.path.join(tmp, "graph.txt")
    G.write_grammar(gp, w.rules)
    G.write_graph(fp, w)
    return gp, fp


def run_comp(grg, *args):
    r = subprocess.run([comp_path(grg)] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    return r.returncode, r.stdout, r.stderr


def final_edges(out):
    return int(re.search(r"^FINAL NUM EDGES: (\d+)$", out, re.M).group(1))


def test_usage_and_unknown_options(grg_mod, tmp_path):
    if not os.path.exists(comp_path(grg_mod)):
        pytest.skip("comp not built")
    rc, _, err = run_comp(grg_mod)
    assert rc == 2 and "usage" in err
    w = G.pointsto(seed=71, num_vars=100, num_edges=200)
    gp, fp = write_inputs(str(tmp_path), w)
    rc, _, err = run_comp(grg_mod, gp, fp, 0, "--bogus")
    assert rc == 2 and "unknown option" in err


@pytest.mark.gpu
def test_in_core_and_stream_output(grg_mod, oracle_mod, tmp_path):
    w = G.pointsto(seed=72, num_vars=800, num_edges=2200)
    gp, fp = write_inputs(str(tmp_path), w)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    out = str(tmp_path / "closure.bin")
    rc, so, se = run_comp(grg_mod, gp, fp, 0, "--out", out)
    assert rc == 0, se
    assert "NUM VERTICES: 800" in so and "FINAL NUM PARTITIONS: 1" in so
    assert final_edges(so) == r.total
    want, wdeg = r.csr5()
    assert np.array_equal(np.fromfile(out, np.uint8), want)
    assert np.array_equal(np.fromfile(out + ".degree", np.uint32), wdeg)


@pytest.mark.gpu
def test_partitioned_checkpoint_and_resume(grg_mod, oracle_mod, tmp_path):
    w = G.alias(seed=73, num_vars=2000, num_base_edges=5000, block=500)
    gp, fp = write_inputs(str(tmp_path), w)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    ck, out = str(tmp_path / "ck.bin"), str(tmp_path / "closure.bin")
    rc, so, se = run_comp(grg_mod, gp, fp, 0, "--partitions", 4, "--checkpoint", ck)
    assert rc == 0, se
    assert "INITIAL NUM PARTITIONS: 4" in so and final_edges(so) == r.total
    # the closed set resumes from the file alone (the graph file is not read again)
    open(fp, "w").write("0\t0\n")
    rc, so2, se = run_comp(grg_mod, gp, fp, 0, "--resume", ck, "--out", out)
    assert rc == 0, se
    assert final_edges(so2) == r.total
    want, wdeg = r.csr5()
    assert np.array_equal(np.fromfile(out, np.uint8), want)
    assert np.array_equal(np.fromfile(out + ".degree", np.uint32), wdeg)


# The reference's own sample (src/inputFiles, run by src/run.sh), copied to tests/fixtures.
SAMPLE_COUNTS = {"M": 0, "DV": 0, "d": 352, "-d": 0, "V": 591, "MAM": 530, "AMs": 591, "MAs": 530,
                 "Mq": 530, "MA": 0, "-a": 0, "AM": 61, "a": 61}


def _sample_paths():
    from conftest import REFERENCE_SAMPLE
    return (os.path.join(REFERENCE_SAMPLE, "rules_pointsto.txt"),
            os.path.join(REFERENCE_SAMPLE, "programGraph_sample_pointsto.txt"))


@pytest.mark.gpu
@pytest.mark.parametrize("parts", [0, 3])
def test_reference_sample_inputs(grg_mod, oracle_mod, tmp_path, parts):
    """`comp` on the reference's sample grammar and graph, argument order as in
    src/run.sh, filter 0: the reference's stdout lines, 3246 closure edges with
    the per-label counts, and the compressed stream byte for byte against the
    oracle's writer (in core and over partitions)."""
    gp, fp = _sample_paths()
    out = str(tmp_path / "closure.bin")
    extra = ["--partitions", parts] if parts else []
    rc, so, se = run_comp(grg_mod, fp, gp, 0, "--out", out, *extra)
    assert rc == 0, se
    assert "NUM RULES: 12" in so and "NUM LABELS: 13" in so
    assert "NUM VERTICES: 530" in so and "INITIAL NUM EDGES: 2000" in so
    assert final_edges(so) == 3246
    got = {m.group(1): int(m.group(2)) for m in re.finditer(r"^LABEL (\S+) EDGES: (\d+)$", so, re.M)}
    assert got == SAMPLE_COUNTS
    g = oracle_mod.parse_grammar(gp)
    nv, s, d, l = oracle_mod.parse_graph(fp, g)
    r = oracle_mod.closure(nv, g.rules, g.num_labels, 0, s, d, l)
    assert r.total == 3246
    want, wdeg = r.csr5()
    assert np.array_equal(np.fromfile(out, np.uint8), want)
    assert np.array_equal(np.fromfile(out + ".degree", np.uint32), wdeg)


@pytest.mark.gpu
def test_reference_sample_edges_through_library(grg_mod, oracle_mod):
    """The same sample through the C ABI: identical sorted edge list and edge-set hash."""
    gp, fp = _sample_paths()
    g = grg_mod.parse_grammar(gp)
    nv, s, d, l = grg_mod.parse_graph(fp, g)
    ctx, st = grg_mod.run_closure(nv, g.rules, g.num_labels, 0, s, d, l, device=0)
    go = oracle_mod.parse_grammar(gp)
    r = oracle_mod.closure(nv, go.rules, go.num_labels, 0, *oracle_mod.parse_graph(fp, go)[1:])
    assert st["total_edges"] == r.total == 3246
    assert ctx.set_hash() == r.set_hash
    for a, b in zip(ctx.export_edges(), r.edges()):
        assert np.array_equal(a, b)
    ctx.close()


@pytest.mark.gpu
def test_reference_sample_filter1_refused(grg_mod):
    """filter 1 on the sample grammar: its binary rules have derivable second
    symbols (AMs ::= AMs AM with AM derived), where the reference's answer
    depends on its partition schedule; comp exits with the filter status."""
    gp, fp = _sample_paths()
    rc, so, se = run_comp(grg_mod, fp, gp, 1)
    assert rc == 1
    assert "filter_flag=1" in se
