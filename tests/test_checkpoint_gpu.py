"""GPU tests of checkpoint / resume of the out-of-core closure (grg_part_save,
grg_part_restore, run budgets) and of the per-partition compressed streams.

An interruption is made on the host: a run budget stops grg_part_run between
device runs (nothing in flight), the checkpoint file is the only thing carried
over, and a fresh context restores it -- as a restarted process would. The
result must equal the uninterrupted closure and the oracle bit for bit."""
import os

import numpy as np
import pytest

import grg_gen as G

pytestmark = pytest.mark.gpu


def oracle_result(O, w, f):
    r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, f, w.src, w.dst, w.lab)
    return [int(x) for x in r.label_counts()], r.set_hash


def new_ctx(grg, w, pool_bytes=0):
    ctx = grg.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    if pool_bytes:
        ctx.set_pool_limit(pool_bytes)
    return ctx


def run_in_slices(grg, w, f, parts, path, budget, pool_bytes=0):
    """Load, then run `budget` device runs per process-like slice: every slice
    restores the checkpoint into a new context. Returns (counts, hash, slices)."""
    ctx = new_ctx(grg, w, pool_bytes)
    p = grg.Partitioned(ctx, w.num_vars, parts)
    p.load_edges(w.src, w.dst, w.lab)
    p.save(path)
    p.close()
    ctx.close()
    slices = 0
    while True:
        ctx = new_ctx(grg, w, pool_bytes)
        p = grg.Partitioned(ctx, 0, 0, restore_from=path)
        p.set_checkpoint(path, 1)
        p.set_run_budget(budget)
        p.run(f)
        slices += 1
        if not p.paused:
            counts, h = p.label_counts()
            p.close()
            ctx.close()
            return [int(x) for x in counts], h, slices
        p.close()
        ctx.close()
        assert slices < 1000


@pytest.mark.parametrize("budget", [1, 3])
def test_pairs_schedule_resumes_across_contexts(grg_mod, oracle_mod, tmp_path, budget):
    w = G.pointsto(seed=61, num_vars=900, num_edges=2400)
    want = oracle_result(oracle_mod, w, 0)
    counts, h, slices = run_in_slices(grg_mod, w, 0, 4, str(tmp_path / "ck.bin"), budget)
    assert (counts, h) == want
    assert slices > 1


def test_stream_schedule_resumes_across_contexts(grg_mod, oracle_mod, tmp_path):
    w = G.dataflow_blocks(seed=62, num_blocks=6, block=500, num_edges=9000)
    want = oracle_result(oracle_mod, w, 1)
    counts, h, slices = run_in_slices(grg_mod, w, 1, 5, str(tmp_path / "ck.bin"), 2)
    assert (counts, h) == want
    assert slices == 3                       # 5 partitions, 2 runs per slice


def test_resume_after_splits(grg_mod, oracle_mod, tmp_path):
    # a pool limit that forces splits: split partitions and their pair history survive the file
    w = G.pointsto(seed=63, num_vars=1200, num_edges=3000)
    want = oracle_result(oracle_mod, w, 0)
    ctx, st = grg_mod.run_closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    pool = st["pool_elems_used"] * 69 // 3
    ctx.close()
    counts, h, slices = run_in_slices(grg_mod, w, 0, 2, str(tmp_path / "ck.bin"), 16, pool_bytes=pool)
    assert (counts, h) == want and slices > 1


def test_paused_run_keeps_its_filter_and_closed_sets_restore(grg_mod, oracle_mod, tmp_path):
    w = G.dataflow_blocks(seed=64, num_blocks=4, block=500, num_edges=6000)
    want = oracle_result(oracle_mod, w, 1)
    path = str(tmp_path / "ck.bin")
    ctx = new_ctx(grg_mod, w)
    p = grg_mod.Partitioned(ctx, w.num_vars, 4)
    p.load_edges(w.src, w.dst, w.lab)
    p.set_checkpoint(path, 0)                # saved only when paused or finished
    p.set_run_budget(1)
    p.run(1)
    assert p.paused
    with pytest.raises(grg_mod.GrgError) as ei:
        p.run(0)                              # continuing with another filter is refused
    assert ei.value.status == grg_mod.E_ARG
    p.set_run_budget(0)
    p.run(1)
    assert not p.paused
    assert ([int(x) for x in p.label_counts()[0]], p.label_counts()[1]) == want
    p.close()
    ctx.close()
    # the final checkpoint is of the closed set: counts without any run
    ctx = new_ctx(grg_mod, w)
    p = grg_mod.Partitioned(ctx, 0, 0, restore_from=path)
    counts, h = p.label_counts()
    assert ([int(x) for x in counts], h) == want
    with pytest.raises(grg_mod.GrgError) as ei:
        p.run(1)
    assert ei.value.status == grg_mod.E_STATE
    p.close()
    ctx.close()


def test_damaged_or_foreign_checkpoints_are_refused(grg_mod, tmp_path):
    w = G.pointsto(seed=65, num_vars=500, num_edges=1300)
    path = str(tmp_path / "ck.bin")
    ctx = new_ctx(grg_mod, w)
    p = grg_mod.Partitioned(ctx, w.num_vars, 3)
    p.load_edges(w.src, w.dst, w.lab)
    p.save(path)
    p.close()
    data = open(path, "rb").read()
    bad = []
    flipped = bytearray(data)
    flipped[len(data) // 2] ^= 0x40
    bad.append(bytes(flipped))                       # one bit changed: checksum
    bad.append(data[: len(data) - 9])                # truncated
    bad.append(data[:40])                            # header only
    bad.append(b"")                                  # empty
    for k, blob in enumerate(bad):
        q = str(tmp_path / f"bad{k}.bin")
        open(q, "wb").write(blob)
        with pytest.raises(grg_mod.GrgError) as ei:
            grg_mod.Partitioned(ctx, 0, 0, restore_from=q)
        assert ei.value.status == grg_mod.E_IO, k
    with pytest.raises(grg_mod.GrgError) as ei:
        grg_mod.Partitioned(ctx, 0, 0, restore_from=str(tmp_path / "missing.bin"))
    assert ei.value.status == grg_mod.E_IO
    ctx.close()
    # a context with another grammar refuses the file
    w2 = G.dataflow_small(seed=66, num_vars=500, num_edges=1500)
    ctx2 = new_ctx(grg_mod, w2)
    with pytest.raises(grg_mod.GrgError) as ei:
        grg_mod.Partitioned(ctx2, 0, 0, restore_from=path)
    assert ei.value.status == grg_mod.E_IO
    ctx2.close()
    assert not os.path.exists(path + ".tmp")


def test_partition_streams_concatenate_to_the_whole(grg_mod, oracle_mod):
    # per-partition spill streams (the reference's Partition<k> files) in bound
    # order are the stream of the whole closed graph
    w = G.alias(seed=67, num_vars=2400, num_base_edges=6000, block=400)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    ctx = new_ctx(grg_mod, w)
    p = grg_mod.Partitioned(ctx, w.num_vars, 5)
    p.load_edges(w.src, w.dst, w.lab)
    p.run(0)
    parts = [p.export_csr5(i) for i in range(len(p.bounds()) - 1)]
    stream = np.concatenate([s for s, _ in parts])
    deg = np.concatenate([d for _, d in parts])
    want, wdeg = r.csr5()
    assert np.array_equal(stream, want) and np.array_equal(deg, wdeg)
    p.close()
    ctx.close()
