"""The bench's multi-rank plumbing on CPU (gloo, world size 2): timings are
reduced to their maximum over the ranks, and the reference arm runs on rank 0
only. The GPU replicas themselves need no exchange (each closes its own graph)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path[:0] = [ROOT]
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 3.5], dist, "cpu")
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 10.0, 3.5]


def test_max_over_ranks_single():
    pytest.importorskip("torch")
    sys.path[:0] = [ROOT]
    import bench
    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]


def test_reference_arm_rank_nonzero_does_nothing(capsys):
    sys.path[:0] = [ROOT]
    import bench

    class A:
        steps, warmup = 1, 0
    bench.run_reference(A(), None, 2, 1)          # rank 1 of 2: returns at once, prints nothing
    assert capsys.readouterr().out == ""
