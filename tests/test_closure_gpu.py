"""GPU parity tests: the CUDA closure engine (through the C ABI) against the
CPU oracle. Integer/bitset work, so every comparison is bit-exact: identical
(src, dst, label) sets, per-label counts and edge-set hashes."""
import json
import os

import numpy as np
import pytest

import grg_gen as G

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def gpu_closure(grg, w, filter_flag=None, pool_bytes=0, timing=False):
    f = w.filter_flag if filter_flag is None else filter_flag
    return grg.run_closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab,
                           pool_bytes=pool_bytes, timing=timing)


def edge_set(s, d, l):
    return set(zip(s.tolist(), d.tolist(), l.tolist()))


def assert_same_as_oracle(grg, O, w, filter_flag=None, pool_bytes=0, edges=True):
    f = w.filter_flag if filter_flag is None else filter_flag
    r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    ctx, st = gpu_closure(grg, w, f, pool_bytes)
    assert st["total_edges"] == r.total
    assert ctx.label_counts().tolist() == r.label_counts().tolist()
    assert ctx.set_hash() == r.set_hash
    if edges:
        gs, gd, gl = ctx.export_edges()
        os_, od, ol = r.edges()
        assert np.array_equal(gl, ol) and np.array_equal(gs, os_) and np.array_equal(gd, od)
    ctx.close()
    return r, st


def test_pointsto_small_exact(grg_mod, oracle_mod):
    assert_same_as_oracle(grg_mod, oracle_mod, G.pointsto(seed=3, num_vars=300, num_edges=700))


def test_pointsto_2000(grg_mod, oracle_mod):
    g = GOLD["pointsto"]
    r, st = assert_same_as_oracle(grg_mod, oracle_mod, G.pointsto(), edges=False)
    assert r.total == g["total"]


@pytest.mark.parametrize("seed", range(24))
def test_random_grammars(grg_mod, oracle_mod, seed):
    w = G.random_grammar_graph(100 + seed, num_vars=200 + 37 * seed, num_edges=400 + 50 * seed,
                               num_labels=3 + seed % 5, num_rules=3 + seed % 7)
    for f in (0, 1):
        try:
            oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
        except oracle_mod.OracleError as e:
            assert e.code == oracle_mod.ORC_E_FILTER
            with pytest.raises(grg_mod.GrgError) as ei:
                gpu_closure(grg_mod, w, f)
            assert ei.value.status == grg_mod.E_FILTER
            continue
        assert_same_as_oracle(grg_mod, oracle_mod, w, f)


def test_dataflow_small_golden(grg_mod):
    """10k vertices, 30k e edges, filter 0 (N ::= N e | e)."""
    g = GOLD["dataflow_small"]
    w = G.dataflow_small()
    ctx, st = gpu_closure(grg_mod, w)
    assert st["total_edges"] == g["total"] == 93_365_096
    assert dict(zip(w.labels, ctx.label_counts().tolist())) == g["labels"]
    assert ctx.set_hash() == g["hash"]


@pytest.mark.parametrize("layout", [0, 1])
def test_dataflow_blocks_scaled_rounds(grg_mod, layout):
    """Filter 1 reads only static right-hand rows, so the GPU's rounds equal the
    oracle's round-synchronous rounds exactly, in either storage layout. With
    every label stored by source the join reads at least the oracle's
    right-hand elements; stored by destination, N is pushed along e's edges."""
    g = GOLD["dataflow_blocks_b100"]
    w = G.dataflow_blocks(num_blocks=100, num_edges=300_000)
    ctx = grg_mod.Context(0)
    ctx.set_layout(layout)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    st = ctx.closure(w.filter_flag)
    assert st["total_edges"] == g["total"]
    assert ctx.set_hash() == g["hash"]
    assert st["rounds"] == g["rounds"] - 1 or st["rounds"] == g["rounds"]
    assert st["delta_elems"] - st["retry_records"] >= 0
    if layout == 0:
        assert st["column_labels"] == 0
        assert st["right_elems"] >= g["right_elems"]
    else:
        assert st["column_labels"] == 1 << w.labels.index("N")
    ctx.close()


def test_dataflow_blocks_full_size(grg_mod):
    """2,000 blocks x 1,000 vertices, 6M e edges, filter 1: the bench workload.
    Checked against the oracle's recorded count and edge-set hash."""
    g = GOLD["dataflow_blocks"]
    w = G.dataflow_blocks()
    assert w.num_edges == g["num_edges"]
    ctx, st = gpu_closure(grg_mod, w)
    assert st["total_edges"] == g["total"] == 1_316_964_027
    assert dict(zip(w.labels, ctx.label_counts().tolist())) == g["labels"]
    assert ctx.set_hash() == g["hash"]


def test_alias_20k(grg_mod, oracle_mod):
    g = GOLD["alias_20k"]
    w = G.alias(num_vars=20_000, num_base_edges=80_000)
    ctx, st = gpu_closure(grg_mod, w)
    assert st["total_edges"] == g["total"]
    assert ctx.set_hash() == g["hash"]
    # the join's work counters: items ORed into the hash instead of a window; a batch of more
    # runs of a row's records than a warp has window slots joins in passes, so no item of a run
    # goes without a window
    assert st["window_out_elems"] < st["right_elems"] * 192
    assert st["window_noslot_items"] == 0


def test_degree_matches_oracle(grg_mod, oracle_mod):
    w = G.pointsto(seed=9, num_vars=500, num_edges=1500)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    e, el = r.degree()
    ctx, _ = gpu_closure(grg_mod, w)
    deg = ctx.degree()
    assert np.array_equal(deg[0], e) and np.array_equal(deg[3], el)
    assert not deg[1].any() and not deg[2].any() and not deg[4].any() and not deg[5].any()
    sub = ctx.degree(100, 199)
    assert np.array_equal(sub[0], e[100:200]) and np.array_equal(sub[3], el[100:200])


def test_tiny_pool_grows(grg_mod, oracle_mod):
    """A pool far too small for the closure forces table growth and pool growth."""
    assert_same_as_oracle(grg_mod, oracle_mod, G.dataflow_small(num_vars=2000, num_edges=6000), pool_bytes=1 << 16,
                          edges=False)


def test_edge_cases(grg_mod, oracle_mod):
    O = oracle_mod
    cases = [
        # (num_vars, rules, num_labels, filter, edges)
        (5, [[1, 0, 0], [2, 1, 0]], 2, 0, []),                          # epsilon + unary, no edges
        (5, [[1, 0, 0], [2, 1, 0]], 2, 1, []),                          # filter 1 drops unary
        (1, [[1, 1, 2], [1, 2, 0]], 2, 0, [(0, 0, 2)]),                 # single vertex self loop
        (3, [[1, 1, 2], [1, 2, 0]], 2, 0, [(0, 1, 2), (0, 1, 2), (1, 2, 2)]),   # duplicate edges collapse
        (400, [[1, 1, 2], [1, 2, 0]], 3, 0, [(i, (i * 7 + 1) % 400, 2) for i in range(400)]),  # unused label 3
        (1000, [[1, 1, 1]], 1, 0, [(i, i + 1, 1) for i in range(999)]),  # transitive chain, 999 rounds
        (193, [[1, 1, 2]], 2, 1, [(i, 192 - i, 2) for i in range(193)] + [(0, 5, 1)]),  # element boundaries
    ]
    for nv, rules, nl, f, edges in cases:
        e = np.array(edges, dtype=np.int64).reshape(-1, 3)
        s, d, l = e[:, 0].astype(np.uint32), e[:, 1].astype(np.uint32), e[:, 2].astype(np.uint8)
        r = O.closure(nv, rules, nl, f, s, d, l)
        ctx, st = grg_mod.run_closure(nv, rules, nl, f, s, d, l)
        assert st["total_edges"] == r.total, (nv, rules, f)
        gs, gd, gl = ctx.export_edges()
        os_, od, ol = r.edges()
        assert np.array_equal(gs, os_) and np.array_equal(gd, od) and np.array_equal(gl, ol)
        ctx.close()


def test_errors_and_state(grg_mod):
    with grg_mod.Context(0) as ctx:
        with pytest.raises(grg_mod.GrgError) as ei:
            ctx.closure(0)
        assert ei.value.status == grg_mod.E_STATE
        with pytest.raises(grg_mod.GrgError) as ei:
            ctx.transfer_rules([[1, 0, 2]], 2)          # RHS2 without RHS1
        assert ei.value.status == grg_mod.E_ARG
        ctx.transfer_rules([[1, 1, 1]], 1)
        ctx.load_edges(4, np.array([0, 1], np.uint32), np.array([1, 2], np.uint32), np.array([1, 1], np.uint8))
        with pytest.raises(grg_mod.GrgError) as ei:
            ctx.closure(1)                              # A ::= A A is schedule-dependent under filter 1
        assert ei.value.status == grg_mod.E_FILTER
        st = ctx.closure(0)
        assert st["total_edges"] == 3
        with pytest.raises(grg_mod.GrgError) as ei:
            ctx.closure(0)
        assert ei.value.status == grg_mod.E_STATE
        # reload on the same context and close again
        ctx.load_edges(4, np.array([0, 1, 2], np.uint32), np.array([1, 2, 3], np.uint32), np.array([1, 1, 1], np.uint8))
        assert ctx.closure(0)["total_edges"] == 6


def test_device_load_equals_host_load(grg_mod):
    torch = pytest.importorskip("torch")
    w = G.dataflow_blocks(num_blocks=30, num_edges=90_000)
    src = torch.from_numpy(w.src.astype(np.int32)).cuda()
    dst = torch.from_numpy(w.dst.astype(np.int32)).cuda()
    lab = torch.from_numpy(w.lab).cuda()
    with grg_mod.Context(0) as ctx:
        ctx.transfer_rules(w.rule_ids(), w.num_labels)
        ctx.set_stream(torch.cuda.current_stream().cuda_stream)
        ctx.load_edges_device(w.num_vars, w.num_edges, src.data_ptr(), dst.data_ptr(), lab.data_ptr())
        a = ctx.closure(1)["total_edges"]
        ha = ctx.set_hash()
    ctx2, st = gpu_closure(grg_mod, w)
    assert a == st["total_edges"] and ha == ctx2.set_hash()


@pytest.mark.parametrize("name", ["pointsto", "alias", "dataflow", "chain"])
def test_device_rounds_equal_host_rounds(grg_mod, oracle_mod, name):
    """Rounds replayed from the CUDA graph's WHILE node give the same closure
    as rounds driven from the host. (How new edges split over rounds depends on
    the timing of a round's concurrent inserts, so round and delta counts may
    differ; the closure may not.)"""
    w = {"pointsto": lambda: G.pointsto(seed=31, num_vars=900, num_edges=2200),
         "alias": lambda: G.alias(seed=32, num_vars=4000, num_base_edges=9000, block=500),
         "dataflow": lambda: G.dataflow_blocks(seed=33, num_blocks=20, block=500, num_edges=30000),
         "chain": lambda: G.random_grammar_graph(34, num_vars=600, num_edges=599, num_labels=2, num_rules=2)}[name]()
    if name == "chain":
        w.rules = [("L0", "L0", "L1"), ("L0", "L1")]
        w.labels = ["L0", "L1"]
        w.src = np.arange(599, dtype=np.uint32)
        w.dst = w.src + 1
        w.lab = np.full(599, 2, np.uint8)
        w.filter_flag = 0
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, w.filter_flag, w.src, w.dst, w.lab)
    out = []
    for dev in (False, True):
        ctx = grg_mod.Context(0)
        ctx.set_device_rounds(dev)
        ctx.transfer_rules(w.rule_ids(), w.num_labels)
        ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
        st = ctx.closure(w.filter_flag)
        out.append((ctx.label_counts().tolist(), ctx.set_hash()))
        ctx.close()
    assert out[0] == out[1]
    assert out[1][0] == r.label_counts().tolist() and out[1][1] == r.set_hash


@pytest.mark.parametrize("name", ["pointsto", "alias", "dataflow"])
def test_join_windows_equal(grg_mod, oracle_mod, name):
    """The narrow (8-element) and wide (12-element) join windows give the oracle's closure."""
    w = {"pointsto": lambda: G.pointsto(seed=41, num_vars=900, num_edges=2200),
         "alias": lambda: G.alias(seed=42, num_vars=4000, num_base_edges=9000, block=700),
         "dataflow": lambda: G.dataflow_blocks(seed=43, num_blocks=20, block=500, num_edges=30000)}[name]()
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, w.filter_flag, w.src, w.dst, w.lab)
    for mode in (0, 1):
        for items in (0, 1):
            ctx = grg_mod.Context(0)
            ctx.set_join_window(mode)
            ctx.set_join_items(items)
            ctx.set_layout(0)              # every label by source: the dataflow closure runs k_join too
            ctx.transfer_rules(w.rule_ids(), w.num_labels)
            ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
            st = ctx.closure(w.filter_flag)
            assert st["wide_window"] == mode
            # the item form applies to labels with a CSR copy, the static second symbols
            # (dataflow: e; points-to: d and -a; alias: d), so each case exercises both forms
            assert st["join_elements"] == items
            assert ctx.label_counts().tolist() == r.label_counts().tolist() and ctx.set_hash() == r.set_hash
            ctx.close()


@pytest.mark.parametrize("device_rounds", [True, False])
def test_tuned_window_measures_then_reuses(grg_mod, oracle_mod, device_rounds):
    """A closure whose degree key must be measured (mode 3 measures even when
    another closure of the process cached the key) times its large first
    round's join pass in both windows (window_tuned 1), and the closure is the
    oracle's despite the extra passes; a mode-2 closure of the same input then
    takes the choice from the cache (window_tuned 2). Fixed modes report 0."""
    w = G.dataflow_blocks(seed=44 + device_rounds, num_blocks=97 + 2 * device_rounds, block=1000,
                          num_edges=291_000 + 6000 * device_rounds)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, w.filter_flag, w.src, w.dst, w.lab)
    want = (r.label_counts().tolist(), r.set_hash)
    seen = []
    for k in range(2):
        ctx = grg_mod.Context(0)
        ctx.set_join_window(3 if k == 0 else 2)
        ctx.set_join_items(3 if k == 0 else 2)
        ctx.set_layout(0)                  # the window is a choice of k_join, which source rows run
        ctx.set_device_rounds(device_rounds)
        ctx.transfer_rules(w.rule_ids(), w.num_labels)
        ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
        st = ctx.closure(w.filter_flag)
        assert (ctx.label_counts().tolist(), ctx.set_hash()) == want
        seen.append((st["window_tuned"], st["wide_window"], st["window_trial_ms"], st["join_elements"],
                     st["items_trial_ms"]))
        ctx.close()
    assert seen[0][0] == 1 and min(seen[0][2]) > 0 and min(seen[0][4]) > 0
    assert seen[1][0] == 2 and seen[1][1] == seen[0][1] and seen[1][2] == [0.0, 0.0]
    assert seen[1][3] == seen[0][3]                  # the item form comes from the cache too
    ctx = grg_mod.Context(0)
    ctx.set_join_window(1)
    ctx.set_join_items(0)
    ctx.set_layout(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    assert ctx.closure(w.filter_flag)["window_tuned"] == 0       # both choices fixed: nothing tuned
    ctx.close()


def test_small_rounds_split_and_retry_overflow(grg_mod, oracle_mod, monkeypatch):
    """Small rounds are joined as sub-records; rows that outgrow their tables make
    joins fail and retry, and with a 16-record retry list the failures overflow
    it, so the round's whole first pass re-runs after the tables grow."""
    monkeypatch.setenv("GRG_RETRY_ROOM", "16")
    cases = [(G.dataflow_small(seed=46, num_vars=3000, num_edges=9000), 0),
             (G.pointsto(seed=45, num_vars=700, num_edges=1800), 0)]
    for w, f in cases:
        r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
        for dev, layout in ((False, 1), (True, 1), (True, 0)):
            ctx = grg_mod.Context(0)
            ctx.set_device_rounds(dev)
            ctx.set_layout(layout)
            ctx.transfer_rules(w.rule_ids(), w.num_labels)
            ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
            st = ctx.closure(f)
            if w.name == "dataflow_small":           # rows of 3000 ids outgrow 16-slot tables
                assert st["retry_records"] > 16 and st["grow_rows"] > 0
            assert ctx.label_counts().tolist() == r.label_counts().tolist() and ctx.set_hash() == r.set_hash
            ctx.close()


@pytest.mark.parametrize("mode", ["0", "1", None])
@pytest.mark.parametrize("name", ["alias", "pointsto", "dataflow"])
def test_insert_modes_equal_oracle(grg_mod, oracle_mod, monkeypatch, name, mode):
    """Joins that write candidates for k_apply (GRG_DIRECT_INSERTS=0) and joins that insert
    directly (1) give the oracle's closure, also with a pool small enough that tables grow and
    inserts fail and re-run; by default a grammar with a derivable right-hand label (alias,
    points-to) inserts directly and the dataflow grammar writes candidates."""
    w = {"alias": lambda: G.alias(seed=71, num_vars=20_000, num_base_edges=80_000, block=500),
         "pointsto": lambda: G.pointsto(seed=72, num_vars=1500, num_edges=5000),
         "dataflow": lambda: G.dataflow_blocks(seed=73, num_blocks=30, num_edges=90_000)}[name]()
    if mode is None:
        monkeypatch.delenv("GRG_DIRECT_INSERTS", raising=False)
    else:
        monkeypatch.setenv("GRG_DIRECT_INSERTS", mode)
    for pool in (0, 1 << 18):
        r, st = assert_same_as_oracle(grg_mod, oracle_mod, w, pool_bytes=pool, edges=False)
        want = (name != "dataflow") if mode is None else mode == "1"
        assert st["direct_inserts"] == want
        assert (st["candidates"] == 0) == want
