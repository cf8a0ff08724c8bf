"""Continuous-batching closure service on one GPU.

Jobs (independent program graphs, each with the dataflow or the alias grammar)
arrive over time. The service admits an arrived job as soon as a job slot, a
vertex range and its projected HBM footprint are available, places it in the
shared engine context (grg_batch_admit) and keeps stepping semi-naive rounds
over every admitted job; a job whose last round had no delta records has
reached its fixpoint, its per-label counts and edge-set hash are read, and its
vertex range is released for the next arrivals. Work of jobs admitted at
different times overlaps on the device, one round at a time.

Reports per-job arrival -> result and admission -> result latencies (p50/p99)
and aggregate closure edges/s over the makespan, and can close the same jobs
one at a time with the plain engine for comparison.
"""
from __future__ import annotations

import collections
import math
import time
from dataclasses import dataclass, field

import numpy as np

import grg
import grg_gen as G

GRAMMARS = [(G.DATAFLOW_RULES, G.grammar_labels(G.DATAFLOW_RULES)),
            (G.ALIAS_RULES, G.grammar_labels(G.ALIAS_RULES))]
KIND = {"dataflow": 0, "alias": 1}
DERIVED = {0: 1, 1: 3}        # derived label tables per vertex for the footprint model


@dataclass
class Job:
    job: int
    kind: str
    num_vars: int
    src: np.ndarray
    dst: np.ndarray
    lab: np.ndarray
    arrival_s: float
    admit_s: float = -1.0
    done_s: float = -1.0
    counts: list = field(default_factory=list)
    hash: int = 0
    slot: int = -1
    base: int = -1

    @property
    def grammar(self):
        return KIND[self.kind]

    @property
    def edges(self):
        return int(sum(self.counts))


def make_jobs(specs, block=1000):
    """Graphs for batch_mix specs: dataflow jobs use the block generator with
    'e' edges only (filter 0 applies N ::= e), alias jobs the block-confined
    alias generator; E = 3..5 x V total edges."""
    jobs = []
    for sp in specs:
        v, e = sp["num_vars"], sp["edges"]
        if sp["kind"] == "dataflow":
            nb = max(1, v // block)
            w = G.dataflow_blocks(seed=sp["seed"] & 0xFFFFFFFF, num_blocks=nb, block=block,
                                  num_edges=max(3 * nb * block, min(e, 5 * nb * block)), seed_n=False)
        else:
            w = G.alias(seed=sp["seed"] & 0xFFFFFFFF, num_vars=v, num_base_edges=max(v, e // 2), block=block)
        jobs.append(Job(sp["job"], sp["kind"], w.num_vars, w.src, w.dst, w.lab, sp["arrival_s"]))
    return jobs


POOL_BYTES_PER_SLOT = 65      # element, delta bitmap, dirty bit (rounded up)


def footprint_bytes(j: Job) -> int:
    """Projected HBM footprint of a job's tables (admission model): its input
    edges twice, 64 slots per vertex and the presized derived rows, at 65 bytes
    per pool slot. plain() reports the pool each job really used, so the model
    can be checked against it."""
    slots = 2 * len(j.src) + j.num_vars * 64 + 16 * DERIVED[j.grammar] * j.num_vars
    return POOL_BYTES_PER_SLOT * slots


class RangeAllocator:
    """First-fit allocator of vertex ranges in [0, size)."""

    def __init__(self, size: int):
        self.free = [(0, size)]

    def alloc(self, n: int):
        for i, (b, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    self.free.pop(i)
                else:
                    self.free[i] = (b + n, ln - n)
                return b
        return None

    def release(self, b: int, n: int):
        self.free.append((b, n))
        self.free.sort()
        merged = []
        for s, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == s:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((s, ln))
        self.free = merged


def serve(jobs, max_vars, max_jobs=256, budget_bytes=None, device=0, realtime=True, rounds_per_step=4,
          drain_rounds=None):
    """Run the service over `jobs` (arrival_s relative to the start). With
    realtime=False every job is available at t=0 (a pure batch). A step runs
    rounds_per_step rounds while jobs wait for admission, else drain_rounds
    (0 = until every admitted job has reached its fixpoint; default: 0 for a
    pure batch, where only throughput counts, and 8 when serving, so that a job
    is reported within a few rounds of its fixpoint). The rounds of a step run
    on the device without host round trips."""
    if drain_rounds is None:
        drain_rounds = 8 if realtime else 0
    ctx = grg.Context(device)
    ctx.allocate_pool(0)
    batch = grg.Batch(ctx, max_vars, max_jobs, GRAMMARS, 0)
    if budget_bytes is None:
        budget_bytes = 1 << 62
    ranges = RangeAllocator(max_vars)
    free_slots = list(range(max_jobs))[::-1]
    pending = collections.deque(sorted(jobs, key=lambda j: j.arrival_s))
    active = {}
    committed = 0
    peak_committed = 0
    held_by_budget = 0           # steps at which an arrived job waited for projected memory
    steps = 0
    t0 = time.perf_counter()
    while pending or active:
        now = time.perf_counter() - t0
        # admit every arrived job that fits (slot, vertex range, projected memory)
        while pending and (not realtime or pending[0].arrival_s <= now) and free_slots:
            j = pending[0]
            fp = footprint_bytes(j)
            if active and committed + fp > budget_bytes:
                held_by_budget += 1
                break
            base = ranges.alloc(j.num_vars)
            if base is None:
                break
            pending.popleft()
            j.slot, j.base = free_slots.pop(), base
            batch.admit(j.slot, base, j.grammar, j.num_vars, j.src, j.dst, j.lab)
            j.admit_s = time.perf_counter() - t0
            if not realtime:
                j.arrival_s = 0.0
            committed += fp
            peak_committed = max(peak_committed, committed)
            active[j.slot] = j
        if not active:
            if pending:
                time.sleep(max(0.0, pending[0].arrival_s - (time.perf_counter() - t0)))
            continue
        rec, _ = batch.step(rounds_per_step if pending else drain_rounds)
        steps += 1
        now = time.perf_counter() - t0
        for slot in [s for s, j in active.items() if rec[s] == 0]:
            j = active.pop(slot)
            cnt, h = batch.result(slot, j.grammar)
            j.counts, j.hash, j.done_s = [int(x) for x in cnt], h, now
            batch.release(slot)
            ranges.release(j.base, j.num_vars)
            free_slots.append(slot)
            committed -= footprint_bytes(j)
    makespan = time.perf_counter() - t0
    ctx.close()
    lat = np.array([j.done_s - j.arrival_s for j in jobs])
    lat_adm = np.array([j.done_s - j.admit_s for j in jobs])
    total = sum(j.edges for j in jobs)
    return {"jobs": len(jobs), "steps": steps, "makespan_s": makespan, "total_edges": total,
            "budget_bytes": budget_bytes, "peak_projected_bytes": peak_committed, "held_by_budget": held_by_budget,
            "edges_per_s": total / makespan if makespan > 0 else 0.0,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "p50_admit_s": float(np.percentile(lat_adm, 50)), "p99_admit_s": float(np.percentile(lat_adm, 99))}


def plain(jobs, device=0):
    """The same jobs closed one at a time with the plain engine (grg_load_edges + grg_closure)."""
    ctx = grg.Context(device)
    ctx.allocate_pool(0)
    out = []
    t0 = time.perf_counter()
    for j in jobs:
        rules, labels = GRAMMARS[j.grammar]
        rid = np.array([[labels.index(x) + 1 for x in r] + [0] * (3 - len(r)) for r in rules], dtype=np.int32)
        ctx.transfer_rules(rid, len(labels))
        ctx.load_edges(j.num_vars, j.src, j.dst, j.lab)
        st = ctx.closure(0)
        out.append((st["total_edges"], [int(x) for x in ctx.label_counts()], ctx.set_hash(),
                    int(st["pool_elems_used"]) * POOL_BYTES_PER_SLOT))
    dt = time.perf_counter() - t0
    ctx.close()
    total = sum(o[0] for o in out)
    return {"seconds": dt, "total_edges": total, "edges_per_s": total / dt if dt > 0 else 0.0, "results": out}
