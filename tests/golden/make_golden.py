"""Generate tests/golden/golden.json: oracle results for the seeded workloads.

    python tests/golden/make_golden.py                 # every entry
    python tests/golden/make_golden.py alias_c3 ...    # only these entries (others kept)

Each entry records the closure of one seeded workload as computed by the CPU
oracle (oracle/grg_oracle.c): total and per-label edge counts, the
order-independent edge-set hash, the number of semi-naive rounds and the
per-round work counters. The GPU tests compare the CUDA engine against these
figures where re-running the oracle would be slow (the 2M-vertex dataflow
workload takes ~25 s on 8 host threads, the 1M-vertex alias closure ~40 s, the
8M-vertex one several minutes and ~30 GB of host memory).

"reference_sample" records the oracle on the reference's own sample inputs
(src/inputFiles, copied to tests/fixtures); its total of 3246 edges matches an
independent pure-Python fixpoint. "batch_mix_sample" records every 16th job
of the 512-job mix (32 jobs, both grammars) closed alone.
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "graspan-g_gb300")]

from oracle import oracle as O  # noqa: E402
import grg_gen as G  # noqa: E402

FIXTURES = os.path.join(ROOT, "tests", "fixtures")
GOLDEN = os.path.join(HERE, "golden.json")

# the 8M-vertex alias workload (out-of-core configuration), as bench.py builds it
C4_ARGS = dict(seed=0x5EED0004, num_vars=8_000_000, num_base_edges=40_000_000, block=1000)
MIX_STRIDE = 16


def record(name, w, with_rounds=False):
    t = time.time()
    r = O.closure(w.num_vars, w.rule_ids(), w.num_labels, w.filter_flag, w.src, w.dst, w.lab)
    st = r.round_stats()
    out = {
        "workload": name,
        "num_vars": int(w.num_vars),
        "num_edges": int(w.num_edges),
        "filter": int(w.filter_flag),
        "total": r.total,
        "labels": dict(zip(w.labels, [int(x) for x in r.label_counts()])),
        "hash": r.set_hash,
        "rounds": r.rounds,
        "new_elems": int(st[:, 1].sum()),
        "left_elems": int(st[:, 2].sum()),
        "right_elems": int(st[:, 3].sum()),
        "meta": w.meta,
    }
    if with_rounds:
        out["round_new_edges"] = [int(x) for x in st[:, 0]]
        out["round_new_elems"] = [int(x) for x in st[:, 1]]
        out["round_left_elems"] = [int(x) for x in st[:, 2]]
        out["round_right_elems"] = [int(x) for x in st[:, 3]]
    print(f"{name}: total={out['total']} rounds={out['rounds']} ({time.time() - t:.1f}s)", flush=True)
    return out


def reference_sample():
    g = O.parse_grammar(os.path.join(FIXTURES, "rules_pointsto.txt"))
    nv, s, d, l = O.parse_graph(os.path.join(FIXTURES, "programGraph_sample_pointsto.txt"), g)
    r = O.closure(nv, g.rules, g.num_labels, 0, s, d, l)
    return {"total": r.total, "labels": dict(zip(g.labels, [int(x) for x in r.label_counts()])),
            "hash": r.set_hash, "rounds": r.rounds, "num_vars": nv, "num_edges": int(len(s))}


def batch_mix_sample():
    """Every MIX_STRIDE-th job of the 512-job mix, closed alone by the oracle."""
    import serve
    specs = G.batch_mix()[::MIX_STRIDE]
    jobs = serve.make_jobs(specs)
    out = []
    t = time.time()
    for sp, j in zip(specs, jobs):
        rules, labels = serve.GRAMMARS[j.grammar]
        rid = [[labels.index(x) + 1 for x in r] + [0] * (3 - len(r)) for r in rules]
        r = O.closure(j.num_vars, rid, len(labels), 0, j.src, j.dst, j.lab)
        out.append({"job": sp["job"], "kind": j.kind, "num_vars": int(j.num_vars), "num_edges": int(len(j.src)),
                    "labels": [int(x) for x in r.label_counts()], "hash": r.set_hash, "total": r.total})
    print(f"batch_mix_sample: {len(out)} jobs, {sum(o['total'] for o in out)} edges ({time.time() - t:.1f}s)",
          flush=True)
    return {"stride": MIX_STRIDE, "jobs": out}


ENTRIES = {
    "reference_sample": reference_sample,
    "dataflow_small": lambda: record("dataflow_small", G.dataflow_small(), True),
    "dataflow_blocks_b100": lambda: record("dataflow_blocks_b100",
                                           G.dataflow_blocks(num_blocks=100, num_edges=300_000), True),
    "dataflow_blocks": lambda: record("dataflow_blocks", G.dataflow_blocks(), True),
    "alias_20k": lambda: record("alias_20k", G.alias(num_vars=20_000, num_base_edges=80_000)),
    "pointsto": lambda: record("pointsto", G.pointsto()),
    "alias_c3": lambda: record("alias_c3", G.alias()),
    "alias_c4": lambda: record("alias_c4", G.alias(**C4_ARGS)),
    "batch_mix_sample": batch_mix_sample,
}


def main(names):
    gold = json.load(open(GOLDEN)) if os.path.exists(GOLDEN) else {}
    for name in names or list(ENTRIES):
        gold[name] = ENTRIES[name]()
        with open(GOLDEN, "w") as f:
            json.dump(gold, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
