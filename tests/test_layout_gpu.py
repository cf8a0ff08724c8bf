"""GPU tests of the storage layouts (grg_set_layout). A derived label whose
rules allow it is stored by destination and its joins are pushes; every result
must be bit-exact with the oracle and with the same closure stored by source:
per-label counts, edge-set hash, the sorted edge list, degrees, element images,
range counts and the compressed stream (the last four read rows by source, so
they first turn the columns around on the device)."""
import numpy as np
import pytest

import grg_gen as G

pytestmark = pytest.mark.gpu


def _closed(grg, w, f, layout):
    ctx = grg.Context(0)
    ctx.set_layout(layout)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    st = ctx.closure(f)
    return ctx, st


CASES = [
    ("dataflow_small_f0", lambda: G.dataflow_small(seed=61, num_vars=3000, num_edges=9000), 0, True),
    ("dataflow_blocks_f1", lambda: G.dataflow_blocks(seed=62, num_blocks=30, num_edges=90_000), 1, True),
    ("dataflow_blocks_f0", lambda: G.dataflow_blocks(seed=63, num_blocks=12, num_edges=36_000, seed_n=False), 0, True),
    ("alias", lambda: G.alias(seed=64, num_vars=4000, num_base_edges=12_000, block=500), 0, False),
    ("pointsto", lambda: G.pointsto(seed=65, num_vars=900, num_edges=2700), 0, False),
]


@pytest.mark.parametrize("name,make,f,columns", CASES, ids=[c[0] for c in CASES])
def test_layouts_equal_oracle(grg_mod, oracle_mod, name, make, f, columns):
    w = make()
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    want_edges = r.edges()
    degs = {}
    for layout in (1, 0):
        ctx, st = _closed(grg_mod, w, f, layout)
        # the dataflow grammar's N is stored by destination under layout 1; alias and
        # points-to grammars have derived second symbols, so nothing is
        n_bit = 1 << (w.labels.index("N")) if "N" in w.labels else 0
        assert st["column_labels"] == (n_bit if (layout == 1 and columns) else 0), (layout, st["column_labels"])
        assert st["total_edges"] == r.total
        assert ctx.label_counts().tolist() == r.label_counts().tolist()
        assert ctx.set_hash() == r.set_hash
        for a, b in zip(ctx.export_edges(), want_edges):
            assert np.array_equal(a, b), layout
        if layout == 1:
            # rows by source after the columns are turned around, on the same context
            deg = ctx.degree(0, w.num_vars - 1)
            wdeg = np.zeros(w.num_vars, np.uint64)
            np.add.at(wdeg, want_edges[0], 1)
            assert np.array_equal(deg[0].astype(np.uint64), wdeg)
            got, gdeg = ctx.export_csr5()
            ws, wd = r.csr5()
            assert np.array_equal(got, ws) and np.array_equal(gdeg, wd)
            V = w.num_vars
            counts, h = ctx.range_counts(V // 3, 2 * V // 3)
            mask = np.zeros(V, np.uint8)
            mask[V // 3:2 * V // 3] = 1
            sel = (want_edges[0] >= V // 3) & (want_edges[0] < 2 * V // 3)
            wc = np.bincount(want_edges[2][sel], minlength=w.num_labels + 1)[1:]
            assert [int(x) for x in counts] == wc.tolist()
            # after the turn-around the counts and hash are unchanged
            assert ctx.label_counts().tolist() == r.label_counts().tolist()
            assert ctx.set_hash() == r.set_hash
        degs[layout] = ctx.degree(0, w.num_vars - 1)
        ctx.close()
    assert np.array_equal(degs[0], degs[1])       # edges and 192-id elements per source row


def test_column_layout_retries_and_host_rounds(grg_mod, oracle_mod, monkeypatch):
    """Pushed joins through the retry path (a tiny pool and a 16-record retry
    list force table growth and whole-pass reruns) and with host-driven rounds."""
    w = G.dataflow_blocks(seed=66, num_blocks=20, num_edges=60_000)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 1, w.src, w.dst, w.lab)
    monkeypatch.setenv("GRG_RETRY_ROOM", "16")
    for rounds in (True, False):
        ctx = grg_mod.Context(0)
        ctx.set_layout(1)
        ctx.set_device_rounds(rounds)
        ctx.allocate_pool(1 << 20)
        ctx.transfer_rules(w.rule_ids(), w.num_labels)
        ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
        st = ctx.closure(1)
        assert st["column_labels"] != 0
        assert st["total_edges"] == r.total and ctx.set_hash() == r.set_hash, rounds
        ctx.close()


@pytest.mark.parametrize("device_rounds", [True, False])
def test_push_kernels_equal_and_tuned(grg_mod, oracle_mod, device_rounds):
    """Both push kernels (one lane per record, edges dealt over the lanes) give the
    oracle's closure; a mode-3 closure times both on its first large round
    (push_tuned 1), a mode-2 closure of the same input takes the cached choice."""
    w = G.dataflow_blocks(seed=67 + device_rounds, num_blocks=97, block=1000, num_edges=291_000)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 1, w.src, w.dst, w.lab)
    want = (r.label_counts().tolist(), r.set_hash)
    seen = []
    for mode in (0, 1, 3, 2):
        ctx = grg_mod.Context(0)
        ctx.set_layout(1)
        ctx.set_push(mode)
        ctx.set_device_rounds(device_rounds)
        ctx.transfer_rules(w.rule_ids(), w.num_labels)
        ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
        st = ctx.closure(1)
        assert (ctx.label_counts().tolist(), ctx.set_hash()) == want, mode
        assert st["column_labels"] != 0
        seen.append((st["push_flat"], st["push_tuned"], st["push_trial_ms"]))
        ctx.close()
    assert seen[0][:2] == (0, 0) and seen[1][:2] == (1, 0)
    assert seen[2][1] == 1 and min(seen[2][2]) > 0
    assert seen[3][1] == 2 and seen[3][0] == seen[2][0]
