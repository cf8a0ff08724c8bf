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
