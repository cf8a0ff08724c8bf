"""GPU test of grg_closure_noalloc, the allocation-free closure entry point.

It exists for callers that cannot allocate device memory while they run (a
serving loop whose memory belongs to another allocator, or a process that
must not let cudaMalloc/cudaFree synchronize the device while other work is
in flight). Its scratch is one static 64 MiB device array shared by every
call, so the test calls it twice in a row on the same input (the second call
must clear what the first left behind) and once on another graph, and checks
each result against the allocating entry points (grg_load_edges +
grg_closure) bit for bit: closure work is integer work, so the tolerance is
exact equality. This file is collected last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import grg_gen as G

pytestmark = pytest.mark.gpu


def _noalloc(lib, torch, w, filter_flag):
    src = torch.from_numpy(w.src.view(np.int32)).cuda()
    dst = torch.from_numpy(w.dst.view(np.int32)).cuda()
    lab = torch.from_numpy(w.lab).cuda()
    counts = torch.full((w.num_labels,), -1, dtype=torch.int64, device="cuda")
    h = torch.zeros(1, dtype=torch.int64, device="cuda")
    rules = np.ascontiguousarray(w.rule_ids().reshape(-1), dtype=np.int32)
    rounds = ctypes.c_uint64()
    torch.cuda.synchronize()
    st = lib.grg_closure_noalloc(0, None, len(rules) // 3, ctypes.c_void_p(rules.ctypes.data), w.num_labels,
                                 filter_flag, w.num_vars, w.num_edges, ctypes.c_void_p(src.data_ptr()),
                                 ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(lab.data_ptr()),
                                 ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(h.data_ptr()),
                                 ctypes.byref(rounds))
    return st, counts.cpu().numpy().view(np.uint64).tolist(), int(h.cpu().numpy().view(np.uint64)[0]), rounds.value


def _allocating(grg, w, filter_flag):
    ctx, st = grg.run_closure(w.num_vars, w.rule_ids(), w.num_labels, filter_flag, w.src, w.dst, w.lab)
    out = ctx.label_counts().tolist(), ctx.set_hash(), st["rounds"]
    ctx.close()
    return out


def test_noalloc_matches_allocating_path_twice(grg_mod):
    torch = pytest.importorskip("torch")
    lib = grg_mod.load_library()
    a = G.pointsto(seed=21, num_vars=800, num_edges=2400)
    b = G.dataflow_blocks(seed=22, num_blocks=6, num_edges=18_000)
    want_a = _allocating(grg_mod, a, 0)
    want_b = _allocating(grg_mod, b, 1)
    for _ in range(2):                              # two calls in a row on the same graph
        st, counts, h, rounds = _noalloc(lib, torch, a, 0)
        assert st == grg_mod.OK, grg_mod.error_string(st)
        assert (counts, h) == (want_a[0], want_a[1])
        assert rounds >= 1
    st, counts, h, rounds = _noalloc(lib, torch, b, 1)   # a different graph and filter reuses the scratch
    assert st == grg_mod.OK
    assert (counts, h, rounds) == want_b
    st, counts, h, _ = _noalloc(lib, torch, a, 0)
    assert st == grg_mod.OK and (counts, h) == (want_a[0], want_a[1])


def test_noalloc_rejects_oversized_graphs(grg_mod):
    torch = pytest.importorskip("torch")
    lib = grg_mod.load_library()
    big = G.dataflow_blocks(seed=3, num_blocks=900, num_edges=90_000)
    # 900k vertices of tables plus 90k edges exceed the 64 MiB scratch: rejected before any launch
    st, counts, _, _ = _noalloc(lib, torch, big, 1)
    assert st == grg_mod.E_RANGE
    assert counts == [2**64 - 1] * big.num_labels       # outputs untouched
    # filter 1 on a schedule-dependent grammar is refused as by grg_closure
    w = G.random_grammar_graph(5, num_vars=50, num_edges=100, num_labels=2, num_rules=1, eps=False, unary=False)
    w.rules = [("L0", "L0", "L0")]
    w.labels = ["L0"]
    w.lab = np.ones(w.num_edges, np.uint8)
    st, _, _, _ = _noalloc(lib, torch, w, 1)
    assert st == grg_mod.E_FILTER


def test_noalloc_refuses_invalid_edges(grg_mod):
    torch = pytest.importorskip("torch")
    lib = grg_mod.load_library()
    w = G.pointsto(seed=49, num_vars=300, num_edges=800)
    good = w.lab.copy()
    w.lab = good.copy()
    w.lab[2] = w.num_labels + 1
    st, counts, _, _ = _noalloc(lib, torch, w, 0)
    assert st == grg_mod.E_LABEL
    w.lab = good
    src = w.src
    w.src = src.copy()
    w.src[9] = w.num_vars
    st, _, _, _ = _noalloc(lib, torch, w, 0)
    assert st == grg_mod.E_RANGE
    w.src = src
    st, counts, h, _ = _noalloc(lib, torch, w, 0)
    assert st == grg_mod.OK and (counts, h) == tuple(_allocating(grg_mod, w, 0)[:2])


def test_noalloc_nomem_then_normal_call(grg_mod):
    """A graph that passes the size check but whose closure outgrows the static
    array (a 20k-vertex dataflow graph whose closure is ~V^2 edges) returns
    GRG_E_NOMEM with the outputs untouched; the next call on a small graph
    starts from a cleared array and matches the allocating path bit for bit."""
    torch = pytest.importorskip("torch")
    lib = grg_mod.load_library()
    big = G.dataflow_small(seed=31, num_vars=20_000, num_edges=60_000)
    st, counts, _, _ = _noalloc(lib, torch, big, 0)
    assert st == grg_mod.E_NOMEM, grg_mod.error_string(st)
    assert counts == [2**64 - 1] * big.num_labels       # outputs untouched
    small = G.pointsto(seed=32, num_vars=500, num_edges=1500)
    want = _allocating(grg_mod, small, 0)
    for _ in range(2):
        st, counts, h, rounds = _noalloc(lib, torch, small, 0)
        assert st == grg_mod.OK
        assert (counts, h, rounds) == want
