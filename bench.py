#!/usr/bin/env python3
"""Benchmark: closure edges/s and time-to-fixpoint of the GB300 engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {grg,reference}]

Workload (one step = one pass of the hot path over one graph): the
block-structured dataflow graph -- 2,000 procedure blocks x 1,000 vertices,
6,000,000 'e' edges plus their 'N' seed copies, grammar N ::= N e | e,
filter_flag 1 -- closed to its fixpoint (1,316,964,027 edges). A step builds
the element tables from the edge arrays already resident in HBM and runs the
semi-naive rounds until no delta remains. L2 is flushed (a 512 MiB write)
before every timed step.

`e2e` runs the same step through the public API from pinned host arrays
(host->device copy of the edges and device->host read of the per-label counts
inside the timed region).

`--impl reference` times the CPU implementation of the path (the oracle port
in oracle/, all host threads) on a bounded sample of the same workload: every
8th procedure block's source rows (rows are independent under filter 1).

Beside the headline, the JSON line carries the other configurations, each
measured on the device with results checked for consistency (skip them with
--quick): `alias_c3` (1M-vertex alias closure), `alias_c4` (8M-vertex alias
closure in-core, and out-of-core over 64 vertex-range partitions staged
through host memory), `stream_c2` (the dataflow closure exported as the
compressed 5-byte-per-edge stream into page-locked host memory and loaded
back), `out_of_core_c2` (the dataflow closure under a pool limit of a quarter
of what it needs in-core, and its checkpoint saved and restored), and
`serving` (the 512-job mix: continuous batching vs one graph at a time).

Multi-GPU: the closure of one graph does not shard without an exchange step,
so N GPUs run N independent replicas (one per rank, weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "graspan-g_gb300")]

import numpy as np  # noqa: E402

# DRAM bytes (read + write) per join pass measured by ncu on the named workload, with the file
# that records the capture
TRAFFIC = {("dataflow", 2000): (559.0e6, "profiles/traffic_dataflow_blocks_2000.md")}
METRIC = "closure_edges_per_sec"
UNIT = "edges/s"
WORKLOAD = ("dataflow_blocks: 2000 blocks x 1000 vertices, 6M 'e' edges + 6M 'N' seeds, "
            "grammar N ::= N e | e, filter_flag 1")
SAMPLE_EVERY = 8


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(values, dist=None, device="cpu"):
    """Each timing's maximum over the ranks (every rank calls it; one all-reduce)."""
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(w, nthreads=None):
    """Oracle port on every SAMPLE_EVERY-th block's source rows, all host threads."""
    from oracle import oracle as O
    O.build()
    nthreads = nthreads or os.cpu_count() or 1
    block = w.meta.get("block", 1000)
    mask = ((np.arange(w.num_vars) // block) % SAMPLE_EVERY == 0).astype(np.uint8)
    t = time.perf_counter()
    r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, w.filter_flag, w.src, w.dst, w.lab,
                  row_mask=mask, nthreads=nthreads)
    dt = time.perf_counter() - t
    total = r.total
    del r
    return {"value": total / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"closure of every {SAMPLE_EVERY}th block's source rows ({int(mask.sum())} rows, "
                      f"{total} edges, {dt:.2f} s)", "seconds": dt, "edges": total}


def run_reference(args, w, world, rank):
    if rank != 0:
        return
    vals = []
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(w)
        if i >= args.warmup:
            vals.append(cb)
    v = statistics.mean(c["value"] for c in vals)
    secs = statistics.mean(c["seconds"] for c in vals)
    last = vals[-1]
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "u32", "data": "synthetic (seeded generator)", "impl": "reference",
           "config": {"workload": WORKLOAD, "num_vars": w.num_vars, "input_edges": w.num_edges,
                      "sample": last["sample"]},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": last["cores"], "kind": "port", "sample": last["sample"]},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def _closure_once(grg, ctx, w, f):
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.load_edges(w.num_vars, w.src, w.dst, w.lab)
    st = ctx.closure(f)
    return st, [int(x) for x in ctx.label_counts()], ctx.set_hash()


def _partitioned(grg, w, f, parts, pool_bytes=0, checkpoint=None):
    """Out-of-core closure; with `checkpoint` (a dict), the closed set is also
    saved to a file and restored into a new context, timed, and the restored
    counts checked."""
    ctx = grg.Context(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    if pool_bytes:
        ctx.set_pool_limit(pool_bytes)
    p = grg.Partitioned(ctx, w.num_vars, parts)
    t = time.perf_counter()
    p.load_edges(w.src, w.dst, w.lab)
    t_load = time.perf_counter() - t
    st = p.run(f)
    counts, h = p.label_counts()
    if checkpoint is not None:
        import tempfile
        fd, path = tempfile.mkstemp(suffix=".grgpart")
        os.close(fd)
        try:
            t = time.perf_counter()
            p.save(path)
            t_save = time.perf_counter() - t
            size = os.path.getsize(path)
            ctx2 = grg.Context(0)
            ctx2.transfer_rules(w.rule_ids(), w.num_labels)
            t = time.perf_counter()
            p2 = grg.Partitioned(ctx2, 0, 0, restore_from=path)
            t_restore = time.perf_counter() - t
            c2, h2 = p2.label_counts()
            p2.close()
            ctx2.close()
        finally:
            os.remove(path)
        assert ([int(x) for x in c2], h2) == ([int(x) for x in counts], h), "restored set differs"
        checkpoint.update({"file_bytes": size, "save_s": t_save, "restore_s": t_restore,
                           "save_gbs": size / t_save / 1e9, "restore_gbs": size / t_restore / 1e9,
                           "restored_counts_identical": True})
    p.close()
    ctx.close()
    return st, [int(x) for x in counts], h, t_load


def _stream_measurement(grg, w, f, counts, h):
    """The closed graph as the compressed edge stream (5 bytes per edge) through
    the C ABI into page-locked host memory, and loaded back into a new context;
    the reloaded graph must close to the same counts and hash."""
    import ctypes
    import torch
    ctx = grg.Context(0)
    ctx.allocate_pool(0)
    _closure_once(grg, ctx, w, f)
    L, V = ctx._L, w.num_vars
    n = ctypes.c_uint64()
    st = L.grg_export_csr5(ctx._h, 0, V, 0, None, None, ctypes.byref(n))
    assert st in (grg.OK, grg.E_RANGE)
    m = n.value
    stream = torch.empty(m * 5, dtype=torch.uint8, pin_memory=True)
    deg = torch.empty(V, dtype=torch.int32, pin_memory=True)
    t0 = time.perf_counter()
    ctx._check(L.grg_export_csr5(ctx._h, 0, V, m, ctypes.c_void_p(stream.data_ptr()), ctypes.c_void_p(deg.data_ptr()),
                                 ctypes.byref(n)), "export_csr5")
    t_export = time.perf_counter() - t0
    ctx.close()
    ctx = grg.Context(0)
    ctx.allocate_pool(0)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    t0 = time.perf_counter()
    ctx._check(L.grg_load_csr5(ctx._h, V, 0, V, ctypes.c_void_p(deg.data_ptr()), m,
                               ctypes.c_void_p(stream.data_ptr()), 0), "load_csr5")
    t_load = time.perf_counter() - t0
    ctx.closure(f)
    same = ([int(x) for x in ctx.label_counts()], ctx.set_hash()) == (counts, h)
    ctx.close()
    assert same, "reloaded stream closes to a different result"
    return {"edges": m, "stream_bytes": m * 5, "export_s": t_export, "load_s": t_load,
            "export_edges_per_s": m / t_export, "load_edges_per_s": m / t_load,
            "export_stream_gbs": m * 5 / t_export / 1e9, "load_stream_gbs": m * 5 / t_load / 1e9,
            "host_memory": "page-locked", "reload_closes_to_same_result": True}


def extra_measurements(args, w2):
    """C3 and C4 (alias, in-core; C4 also out-of-core over 64 partitions), the
    C2 closure as the compressed edge stream (export and reload), and the C2
    dataflow closure out-of-core under a pool limit."""
    import grg
    import grg_gen as G
    out = {}
    # C3: 1M-vertex alias graph, block-confined locality
    w = G.alias()
    ctx = grg.Context(0)
    ctx.allocate_pool(0)
    _closure_once(grg, ctx, w, 0)                       # warm-up (pool and buffers sized)
    st, c3_counts, c3_hash = _closure_once(grg, ctx, w, 0)
    ctx.close()
    out["alias_c3"] = {"workload": "alias grammar, 1M vertices, 4M base + 4M inverse edges, Zipf(1.8) cap 256, "
                                   "1000-vertex blocks", "closure_edges": st["total_edges"],
                       "time_to_fixpoint_ms": st["closure_ms"], "rounds": st["rounds"],
                       "value": st["total_edges"] / (st["closure_ms"] * 1e-3), "unit": UNIT}
    del w
    # C4: 8M vertices, 40M base + 40M inverse edges; in-core, then 64 partitions through host memory
    w = G.alias(seed=0x5EED0004, num_vars=8_000_000, num_base_edges=40_000_000, block=1000)
    ctx = grg.Context(0)
    ctx.allocate_pool(0)
    st, c4_counts, c4_hash = _closure_once(grg, ctx, w, 0)
    ctx.close()
    pst, p_counts, p_hash, t_load = _partitioned(grg, w, 0, 64)
    assert (p_counts, p_hash) == (c4_counts, c4_hash), "partitioned C4 differs from in-core"
    out["alias_c4"] = {"workload": "alias grammar, 8M vertices, 40M base + 40M inverse edges, 1000-vertex blocks",
                       "closure_edges": st["total_edges"], "in_core_ms": st["closure_ms"], "rounds": st["rounds"],
                       "value": st["total_edges"] / (st["closure_ms"] * 1e-3), "unit": UNIT,
                       "pool_elems_used": st["pool_elems_used"],
                       "out_of_core": {"partitions": pst["num_parts"], "schedule": pst["schedule"],
                                       "runs": pst["runs"], "pairs_skipped": pst["skipped"],
                                       "supersteps": pst["supersteps"], "load_s": t_load, "run_ms": pst["ms"],
                                       "h2d_bytes": pst["h2d_bytes"], "d2h_bytes": pst["d2h_bytes"],
                                       "phase_ms": {k: pst[k] for k in ("stage_ms", "load_ms", "closure_ms",
                                                                        "export_ms", "count_ms")},
                                       "prefetched": pst["prefetched"], "prefetch_hits": pst["prefetch_hits"],
                                       "value": pst["total_edges"] / (pst["ms"] * 1e-3), "unit": UNIT,
                                       "identical_to_in_core": True}}
    del w
    # C4 with 2% of the calls going to the partner block 125 blocks (one partition) away, so the
    # pairs schedule runs cross pairs
    w = G.alias(seed=0x5EED0006, num_vars=8_000_000, num_base_edges=40_000_000, block=1000, partner=125)
    ctx = grg.Context(0)
    ctx.allocate_pool(0)
    st, x_counts, x_hash = _closure_once(grg, ctx, w, 0)
    ctx.close()
    pst, p_counts, p_hash, t_load = _partitioned(grg, w, 0, 64)
    assert (p_counts, p_hash) == (x_counts, x_hash), "partitioned C4 with cross calls differs from in-core"
    out["alias_c4_cross"] = {"workload": "alias grammar, 8M vertices, 40M base + 40M inverse edges, 1000-vertex "
                                         "blocks, 2% of calls to the partner block one partition away",
                             "closure_edges": st["total_edges"], "in_core_ms": st["closure_ms"],
                             "out_of_core": {"partitions": pst["num_parts"], "runs": pst["runs"],
                                             "pairs_skipped": pst["skipped"], "supersteps": pst["supersteps"],
                                             "run_ms": pst["ms"],
                                             "phase_ms": {k: pst[k] for k in ("stage_ms", "load_ms", "closure_ms",
                                                                              "export_ms", "count_ms")},
                                             "prefetched": pst["prefetched"], "prefetch_hits": pst["prefetch_hits"],
                                             "identical_to_in_core": True}}
    del w
    # C2 out-of-core: a pool limit of a quarter of what the in-core closure used
    ctx = grg.Context(0)
    ctx.allocate_pool(0)
    st, c2_counts, c2_hash = _closure_once(grg, ctx, w2, w2.filter_flag)
    ctx.close()
    out["stream_c2"] = dict(workload=WORKLOAD, **_stream_measurement(grg, w2, w2.filter_flag, c2_counts, c2_hash))
    limit = st["pool_elems_used"] * 69 // 4
    ck = {}
    pst, p_counts, p_hash, t_load = _partitioned(grg, w2, w2.filter_flag, 4, limit, checkpoint=ck)
    assert (p_counts, p_hash) == (c2_counts, c2_hash), "partitioned C2 differs from in-core"
    out["out_of_core_c2"] = {"workload": WORKLOAD, "pool_limit_bytes": limit, "partitions": pst["num_parts"],
                             "splits": pst["splits"], "schedule": pst["schedule"], "runs": pst["runs"],
                             "load_s": t_load, "run_ms": pst["ms"],
                             "value": pst["total_edges"] / (pst["ms"] * 1e-3), "unit": UNIT,
                             "identical_to_in_core": True, "checkpoint": ck}
    return out


def serving_measurement(args):
    """Config-5 style mix (half dataflow, half alias; Poisson arrivals at 200/s):
    the continuous-batching service vs the same jobs closed one at a time."""
    import serve
    import grg_gen as G
    specs = G.batch_mix(jobs=args.serve_jobs, vmax=args.serve_vmax)
    jobs = serve.make_jobs(specs)
    # vertex space for the whole mix (HBM holds it: tables take ~250 B per vertex of the union grammar)
    max_vars = min(sum(j.num_vars for j in jobs) + args.serve_vmax, 32_000_000)
    max_jobs = min(len(jobs), 512)
    import torch
    free, _ = torch.cuda.mem_get_info()
    budget = free // 4             # admission by projected footprint binds: a quarter of free HBM
    batched = serve.serve(jobs, max_vars=max_vars, max_jobs=max_jobs, realtime=False)  # all jobs available at t=0
    served = serve.serve(jobs, max_vars=max_vars, max_jobs=max_jobs, realtime=True,    # Poisson arrivals
                         budget_bytes=budget)
    plain = serve.plain(jobs)
    assert served["total_edges"] == plain["total_edges"] == batched["total_edges"]
    # the admission model against the pool each job used when closed alone
    ratio = np.array([serve.footprint_bytes(j) / max(r[3], 1) for j, r in zip(jobs, plain["results"])])
    under = int((ratio < 1.0).sum())
    return {"workload": f"{args.serve_jobs} jobs, V log-uniform 1000..{args.serve_vmax}, edges 3-5 x V, "
                        "half dataflow (block generator, filter 0), half alias (block-confined); Poisson 200 jobs/s",
            "batched_edges_per_s": batched["edges_per_s"], "batched_seconds": batched["makespan_s"],
            "speedup_batched_vs_plain": batched["edges_per_s"] / plain["edges_per_s"] if plain["edges_per_s"] else None,
            "served_edges_per_s": served["edges_per_s"], "served_makespan_s": served["makespan_s"],
            "p50_s": served["p50_s"], "p99_s": served["p99_s"], "p50_admit_s": served["p50_admit_s"],
            "p99_admit_s": served["p99_admit_s"], "plain_edges_per_s": plain["edges_per_s"],
            "served_budget_bytes": served["budget_bytes"], "served_peak_projected_bytes": served["peak_projected_bytes"],
            "served_admissions_held_by_budget": served["held_by_budget"],
            "footprint_model_vs_pool_used": {"min": float(ratio.min()), "p50": float(np.median(ratio)),
                                             "max": float(ratio.max()), "jobs_under_projected": under},
            "plain_seconds": plain["seconds"], "total_edges": served["total_edges"]}


def _oracle_alg_elems(args, w):
    """Join-pass elements (left + right + written) the oracle counted for this
    workload, when tests/golden/golden.json records it (the 2,000-block dataflow
    closure and the 100-block one)."""
    gp = os.path.join(ROOT, "tests", "golden", "golden.json")
    if args.workload != "dataflow" or not os.path.exists(gp):
        return None
    name = {2000: "dataflow_blocks", 100: "dataflow_blocks_b100"}.get(args.blocks)
    g = json.load(open(gp)).get(name) if name else None
    if not g or g.get("num_edges") != int(w.num_edges) or g.get("num_vars") != int(w.num_vars):
        return None
    return g["left_elems"] + g["right_elems"] + g["new_elems"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="grg", choices=["grg", "reference"])
    ap.add_argument("--blocks", type=int, default=2000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--pool-gb", type=float, default=0.0, help="initial element pool (0 = 1/8 of free memory)")
    ap.add_argument("--serve-jobs", type=int, default=512,
                    help="jobs of the served mix (0 = skip the serving measurement)")
    ap.add_argument("--serve-vmax", type=int, default=200000, help="largest job of the served mix")
    ap.add_argument("--quick", action="store_true",
                    help="headline only: skip the other configurations and the serving mix")
    ap.add_argument("--workload", default="dataflow", choices=["dataflow", "alias"],
                    help="dataflow: the headline; alias: the 1M-vertex alias closure alone (for profiling; "
                         "implies --quick and --no-cpu-baseline)")
    ap.add_argument("--alias-vars", type=int, default=1_000_000,
                    help="vertices of the alias workload (4 base edges per vertex; smaller for profiler captures)")
    args = ap.parse_args()
    world, rank, local = dist_setup(args)

    import grg_gen as G
    global WORKLOAD
    if args.workload == "alias" and args.impl == "reference":
        ap.error("--workload alias is a GPU profiling case; the reference arm runs the headline workload")
    if args.workload == "alias":
        WORKLOAD = (f"alias grammar, {args.alias_vars} vertices, {4 * args.alias_vars} base + inverse edges, "
                    "Zipf(1.8) cap 256, 1000-vertex blocks, filter_flag 0")
        w = G.alias(num_vars=args.alias_vars, num_base_edges=4 * args.alias_vars)
        args.quick = args.no_cpu_baseline = True
    else:
        edges = 6_000_000 * args.blocks // 2000
        w = G.dataflow_blocks(num_blocks=args.blocks, num_edges=edges)
    if args.impl == "reference":
        run_reference(args, w, world, rank)
        return

    import torch
    import grg
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    ctx = grg.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.transfer_rules(w.rule_ids(), w.num_labels)
    ctx.allocate_pool(int(args.pool_gb * (1 << 30)))
    d_src = torch.from_numpy(w.src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(w.dst.view(np.int32)).cuda()
    d_lab = torch.from_numpy(w.lab).cuda()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def step(timing):
        ctx.set_kernel_timing(timing)
        ctx.load_edges_device(w.num_vars, w.num_edges, d_src.data_ptr(), d_dst.data_ptr(), d_lab.data_ptr())
        return ctx.closure(w.filter_flag)

    warm = [step(False) for _ in range(args.warmup)]
    # timed device-resident steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    barrier()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            stats.append(step(True))
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = statistics.mean(step_ms)
    total = stats[-1]["total_edges"]
    # e2e through the public API from pinned host memory
    h_src = torch.from_numpy(w.src.view(np.int32)).pin_memory()
    h_dst = torch.from_numpy(w.dst.view(np.int32)).pin_memory()
    h_lab = torch.from_numpy(w.lab).pin_memory()
    lib = grg.load_library()
    import ctypes
    counts = np.zeros(w.num_labels, np.uint64)
    e2e_ms = []
    for i in range(args.steps + 1):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        st = lib.grg_load_edges(ctx._h, w.num_vars, w.num_edges, ctypes.c_void_p(h_src.data_ptr()),
                                ctypes.c_void_p(h_dst.data_ptr()), ctypes.c_void_p(h_lab.data_ptr()), 0)
        assert st == 0, st
        ctx.closure(w.filter_flag)
        counts[:] = ctx.label_counts()
        dt = time.perf_counter() - t
        if i > 0:
            e2e_ms.append(dt * 1e3)
    assert int(counts.sum()) == total
    # max over ranks
    ms_max, e2e_max = max_over_ranks([ms, statistics.mean(e2e_ms)], dist, "cuda")
    if rank == 0:
        hbm, peak_kind = peaks()
        s = stats[-1]
        # algorithmic bytes of the join pass (32 B per 192-id element): left elements +
        # right elements + elements written, in the reference's element unit and its
        # source-row formulation, as the oracle counts them for this workload (recorded
        # in tests/golden/golden.json); the engine's own counters measure its pushes
        # instead when a label is stored by destination, so they serve only as a
        # fallback for workloads without a recorded count and a source-row layout
        alg = _oracle_alg_elems(args, w)
        if alg is None and not s["column_labels"]:
            alg = s["left_elems"] + s["right_elems"] + s["out_elems"]
        alg_bytes = 32.0 * alg if alg is not None else None
        join_ms = statistics.mean(x["join_ms"] for x in stats)
        launches = s["rounds"]
        achieved = alg_bytes / (join_ms * 1e-3) / 1e9 if (join_ms > 0 and alg_bytes) else None
        # DRAM bytes per join pass (k_join + k_apply) of the headline closure, from a one-pass
        # ncu capture of every launch of one closure (profiles/traffic_dataflow_blocks_2000.md);
        # other workloads have no capture
        traffic = TRAFFIC.get((args.workload, args.blocks)) if not s["column_labels"] else None
        cb = None if args.no_cpu_baseline else cpu_baseline(w)
        # the other configurations run once, on a single GPU (replica runs hold every GPU meanwhile)
        single = world == 1 and not args.quick
        serving = serving_measurement(args) if (args.serve_jobs > 0 and single) else None
        extras = extra_measurements(args, w) if single else {}
        out = {
            "metric": METRIC, "value": world * total / (ms_max * 1e-3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD, "num_vars": w.num_vars, "input_edges": w.num_edges,
                       "closure_edges": total, "rounds": s["rounds"], "parallelism": f"replicas{world}",
                       "l2_flush": "512 MiB write before every timed step", "time_to_fixpoint_ms": ms_max,
                       "closure_ms": statistics.mean(x["closure_ms"] for x in stats),
                       "gather_ms": statistics.mean(x["gather_ms"] for x in stats),
                       "join_launches": s["join_launches"], "retry_records": s["retry_records"],
                       "grow_rows": s["grow_rows"], "delta_elems": s["delta_elems"],
                       "pool_elems_used": s["pool_elems_used"],
                       "join_window": ("wide (12 elements)" if s["wide_window"] else "narrow (8 elements)") +
                       {0: ", fixed", 1: ", measured in this step", 2: ", tuned (degree-key cache)"}[
                           int(s["window_tuned"])],
                       "join_items": "table elements" if s["join_elements"] else "destination ids",
                       # one closure's join work: (record, rule) pairs, right-hand elements read, the
                       # items ORed into the hash accumulator instead of a dense window, new elements
                       "join_work": {"left_records": s["left_elems"], "right_elems": s["right_elems"],
                                     "hash_items": s["window_out_elems"],
                                     "hash_items_no_slot": s["window_noslot_items"], "out_elems": s["out_elems"],
                                     "candidates": s["candidates"], "join_inserts": s["join_inserts"],
                                     "direct_inserts": bool(s["direct_inserts"])},
                       # the first closure's trial passes (ms): windows [narrow, wide], item forms [ids, elements]
                       "tuner_trials_ms": warm and {"window": [round(x, 3) for x in warm[0]["window_trial_ms"]],
                                                    "items": [round(x, 3) for x in warm[0]["items_trial_ms"]]},
                       # per-phase join cycles (record load, unary, binary join, flush, retry list): only
                       # in builds with -DGRG_PHASE_TIMERS
                       "join_phase_cycles": s["join_phase_cycles"] if any(s["join_phase_cycles"]) else None,
                       "push_kernel": (("edges dealt over lanes" if s["push_flat"] else "one lane per record")
                                       if s["column_labels"] else None)},
            "e2e": {"value": world * total / (e2e_max * 1e-3), "unit": UNIT,
                    "h2d_bytes_per_step": int(w.num_edges * 9), "d2h_bytes_per_step": int(w.num_labels * 8)},
            "roofline": {"bound": "hbm",
                         "kernel": "join pass (" + ("k_push" if s["column_labels"] else "k_join + k_apply") + ")",
                         "achieved": achieved, "peak": hbm,
                         "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": (achieved / hbm) if achieved else None,
                         "traffic": traffic and traffic[0],
                         "traffic_source": traffic and traffic[1],
                         "alg_bytes_per_launch": alg_bytes / launches if alg_bytes else None,
                         "alg_bytes_source": "oracle counts of the workload" if _oracle_alg_elems(args, w) else
                         "engine counters", "launches_per_step": launches, "join_ms_per_step": join_ms,
                         "layout": "N stored by destination (pushed joins)" if s["column_labels"] else
                         "every label stored by source"},
            "cpu_baseline": cb and {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "clocks": clk.summary(),
            "gpu_launches": int(sum(x["kernel_launches"] for x in stats)),
            "serving": serving,
            **extras,
            "wall_s_timed": t_wall,
        }
        print(json.dumps(out), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
