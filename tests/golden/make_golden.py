"""Generate tests/golden/golden.json: oracle results for the seeded workloads.

    python tests/golden/make_golden.py

Each entry records the closure of one seeded workload as computed by the CPU
oracle (oracle/grg_oracle.c): total and per-label edge counts, the
order-independent edge-set hash, the number of semi-naive rounds and the
per-round work counters. The GPU tests compare the CUDA engine against these
figures where re-running the oracle would be slow (the 2M-vertex dataflow
workload takes ~25 s on 8 host threads).

When the reference checkout is present, the entry "reference_sample" records
the oracle on the reference's own sample inputs (src/inputFiles); its total of
3246 edges matches an independent pure-Python fixpoint.
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

REF = "/root/reference/src/inputFiles"


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


def main():
    gold = {}
    if os.path.isdir(REF):
        g = O.parse_grammar(os.path.join(REF, "rules_pointsto.txt"))
        nv, s, d, l = O.parse_graph(os.path.join(REF, "programGraph_sample_pointsto.txt"), g)
        r = O.closure(nv, g.rules, g.num_labels, 0, s, d, l)
        gold["reference_sample"] = {"total": r.total, "labels": dict(zip(g.labels, [int(x) for x in r.label_counts()])),
                                    "hash": r.set_hash, "rounds": r.rounds, "num_vars": nv, "num_edges": int(len(s))}
    gold["dataflow_small"] = record("dataflow_small", G.dataflow_small(), True)
    gold["dataflow_blocks_b100"] = record("dataflow_blocks_b100", G.dataflow_blocks(num_blocks=100, num_edges=300_000), True)
    gold["dataflow_blocks"] = record("dataflow_blocks", G.dataflow_blocks(), True)
    gold["alias_20k"] = record("alias_20k", G.alias(num_vars=20_000, num_base_edges=80_000))
    gold["pointsto"] = record("pointsto", G.pointsto())
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1)


if __name__ == "__main__":
    main()
