"""GPU tests of contexts with different grammars used together. Each context
carries its own rule table into every launch, so a batch, a plain closure on a
second context and the allocation-free entry point can be interleaved on one
device, and two contexts can close graphs of different grammars at the same
time on their own streams. Every result is compared with the oracle bit for
bit (per-label counts and edge-set hash)."""
import ctypes
import threading

import numpy as np
import pytest

import grg_gen as G
import serve

pytestmark = pytest.mark.gpu


def _oracle(O, w, f=0):
    r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    return [int(x) for x in r.label_counts()], r.set_hash


def _job_oracle(O, j):
    rules, labels = serve.GRAMMARS[j.grammar]
    rid = np.array([[labels.index(x) + 1 for x in r] + [0] * (3 - len(r)) for r in rules], dtype=np.int32)
    r = O.closure(j.num_vars, rid, len(labels), 0, j.src, j.dst, j.lab)
    return [int(x) for x in r.label_counts()], r.set_hash


def _noalloc(lib, torch, w, f):
    src = torch.from_numpy(w.src.view(np.int32)).cuda()
    dst = torch.from_numpy(w.dst.view(np.int32)).cuda()
    lab = torch.from_numpy(w.lab).cuda()
    counts = torch.zeros((w.num_labels,), dtype=torch.int64, device="cuda")
    h = torch.zeros(1, dtype=torch.int64, device="cuda")
    rules = np.ascontiguousarray(w.rule_ids().reshape(-1), dtype=np.int32)
    rounds = ctypes.c_uint64()
    torch.cuda.synchronize()
    st = lib.grg_closure_noalloc(0, None, len(rules) // 3, ctypes.c_void_p(rules.ctypes.data), w.num_labels, f,
                                 w.num_vars, w.num_edges, ctypes.c_void_p(src.data_ptr()),
                                 ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(lab.data_ptr()),
                                 ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(h.data_ptr()),
                                 ctypes.byref(rounds))
    return st, counts.cpu().numpy().view(np.uint64).tolist(), int(h.cpu().numpy().view(np.uint64)[0])


def test_batch_plain_and_noalloc_interleaved(grg_mod, oracle_mod):
    """Steps of a batch over the union of the dataflow and alias grammars, with
    a plain closure of a points-to graph on a second context and an
    allocation-free closure of another points-to graph between the steps."""
    torch = pytest.importorskip("torch")
    lib = grg_mod.load_library()
    jobs = serve.make_jobs(G.batch_mix(seed=91, jobs=6, vmin=500, vmax=3000), block=250)
    ctx = grg_mod.Context(0)
    ctx.allocate_pool(0)
    b = grg_mod.Batch(ctx, sum(j.num_vars for j in jobs) + 1, len(jobs), serve.GRAMMARS, 0)
    base = 0
    for k, j in enumerate(jobs):
        b.admit(k, base, j.grammar, j.num_vars, j.src, j.dst, j.lab)
        base += j.num_vars
    other = grg_mod.Context(0)
    p1 = G.pointsto(seed=92, num_vars=700, num_edges=2100)
    p2 = G.pointsto(seed=93, num_vars=600, num_edges=1900)
    want_p1, want_p2 = _oracle(oracle_mod, p1), _oracle(oracle_mod, p2)
    done = {}
    for step in range(1000):
        rec, _ = b.step(1)
        if step % 2 == 0:
            other.transfer_rules(p1.rule_ids(), p1.num_labels)
            other.load_edges(p1.num_vars, p1.src, p1.dst, p1.lab)
            other.closure(0)
            assert ([int(x) for x in other.label_counts()], other.set_hash()) == want_p1
        else:
            st, counts, h = _noalloc(lib, torch, p2, 0)
            assert st == grg_mod.OK and (counts, h) == want_p2
        for k in range(len(jobs)):
            if k not in done and rec[k] == 0:
                done[k] = b.result(k, jobs[k].grammar)
        if len(done) == len(jobs):
            break
    assert len(done) == len(jobs)
    for k, j in enumerate(jobs):
        counts, h = done[k]
        assert ([int(x) for x in counts], h) == _job_oracle(oracle_mod, j), (k, j.kind)
    other.close()
    ctx.close()


def test_two_contexts_concurrently(grg_mod, oracle_mod):
    """Two host threads, each with its own context and stream, close graphs of
    different grammars (alias, and dataflow under filter 1) at the same time."""
    wa = G.alias(seed=94, num_vars=30_000, num_base_edges=100_000, block=500)
    wd = G.dataflow_blocks(seed=95, num_blocks=40, num_edges=120_000)
    want = {"a": _oracle(oracle_mod, wa, 0), "d": _oracle(oracle_mod, wd, 1)}
    got, errors = {}, []

    def run(name, w, f):
        try:
            ctx = grg_mod.Context(0)
            ctx.allocate_pool(1 << 30)
            res = []
            for _ in range(3):
                ctx.transfer_rules(w.rule_ids(), w.num_labels)
                ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
                ctx.closure(f)
                res.append(([int(x) for x in ctx.label_counts()], ctx.set_hash()))
            ctx.close()
            got[name] = res
        except Exception as e:          # reported by the main thread
            errors.append(e)

    ts = [threading.Thread(target=run, args=("a", wa, 0)), threading.Thread(target=run, args=("d", wd, 1))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for name in ("a", "d"):
        assert got[name] == [want[name]] * 3, name
