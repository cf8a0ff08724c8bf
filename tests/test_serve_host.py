"""CPU tests of the serving host logic (no GPU)."""
import numpy as np

import grg_gen as G
import serve


def test_range_allocator_first_fit_and_merge():
    ra = serve.RangeAllocator(100)
    a = ra.alloc(30)
    b = ra.alloc(30)
    c = ra.alloc(30)
    assert (a, b, c) == (0, 30, 60)
    assert ra.alloc(20) is None
    ra.release(b, 30)
    assert ra.alloc(40) is None
    ra.release(a, 30)
    assert ra.free[0] == (0, 60)          # merged
    assert ra.alloc(50) == 0
    ra.release(0, 50)
    ra.release(c, 30)
    assert ra.free == [(0, 100)]


def test_make_jobs_and_footprint():
    specs = G.batch_mix(seed=3, jobs=6, vmin=300, vmax=2000)
    jobs = serve.make_jobs(specs, block=250)
    assert [j.kind for j in jobs] == ["dataflow", "alias"] * 3
    for j in jobs:
        assert j.src.max() < j.num_vars and j.dst.max() < j.num_vars
        assert 3 <= len(j.src) / j.num_vars <= 10
        assert serve.footprint_bytes(j) > 65 * 64 * j.num_vars
    assert all(np.diff([j.arrival_s for j in jobs]) > 0)


def test_dense_block_graphs_generate():
    """5 x V edges on 1000-vertex blocks ask for more cross-block edges than the
    exits can hold; the generator moves the excess to intra-block edges."""
    w = G.dataflow_blocks(seed=9, num_blocks=4, num_edges=20_000, seed_n=False)
    assert 19_000 <= w.num_edges <= 20_000
    e = w.src.astype(np.int64)
    cross = (e // 1000) != (w.dst.astype(np.int64) // 1000)
    assert cross.sum() <= 4 * 10 * 50
    jobs = serve.make_jobs(G.batch_mix(seed=4, jobs=6, vmin=1000, vmax=5000))
    assert len(jobs) == 6
