"""Seeded synthetic program graphs and grammars for the closure workloads.

Graphs are written in the reference's text format (src/main.cpp:106-139,
177-221): comment lines start with '#', the first data line is
"numEdges\\tnumVars", then numEdges lines "src\\tdst\\tlabel", sorted by src
(the reference's loader requires that order, src/main.cpp:125-129, 202-204).

Workloads (64-bit seed per workload):
  dataflow_small  10,000 vertices, 30,000 'e' edges, grammar N ::= N e | e,
                  filter 0. Out-degree Zipf(2.0) capped at 64; dst within
                  +-256 of src with probability 0.8, else uniform.
  dataflow_blocks 2,000 blocks x 1,000 vertices, 6,000,000 'e' edges, filter
                  1, so the generator also emits an 'N' seed copy of every 'e'
                  edge (filter 1 never applies N ::= e). 85% of edges are
                  intra-block and follow the dataflow_small locality model
                  confined to the block body (its first 990 vertices); the
                  other 15% link a block's last 10 vertices (the exits, which
                  have no intra-block in-edges) to the first 10 vertices of
                  one of the next 5 blocks (mod the number of blocks). This
                  calibration keeps the closure near 1e9 edges (1.3e9).
  alias           V ::= a | a_bar | M | V V ; M ::= d_bar T ; T ::= V d, with
                  an inverse x_bar(dst,src) for every base a/d edge. 60% a,
                  40% d; out-degree Zipf(1.8) capped at 256; locality as
                  dataflow_small, confined to 1,000-vertex procedure blocks
                  (unconfined, every vertex joins one V class and the closure
                  is ~V^2: 1e12 edges at 1M vertices).
  pointsto        the points-to grammar of the reference's sample (epsilon,
                  unary and binary rules) over a seeded a/d graph.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

DATAFLOW_RULES = [("N", "N", "e"), ("N", "e")]
ALIAS_RULES = [("V", "a"), ("V", "a_bar"), ("V", "M"), ("V", "V", "V"), ("M", "d_bar", "T"), ("T", "V", "d")]


@dataclass
class Workload:
    name: str
    num_vars: int
    rules: list                 # tuples of label names (LHS first)
    filter_flag: int
    src: np.ndarray
    dst: np.ndarray
    labels: list                # label name per label id - 1 (grammar first-appearance order)
    lab: np.ndarray             # uint8 label ids (1-based)
    meta: dict = field(default_factory=dict)

    @property
    def num_labels(self):
        return len(self.labels)

    @property
    def num_edges(self):
        return int(self.src.shape[0])

    def rule_ids(self) -> np.ndarray:
        out = np.zeros((len(self.rules), 3), dtype=np.int32)
        for i, r in enumerate(self.rules):
            for j, name in enumerate(r):
                out[i, j] = self.labels.index(name) + 1
        return out


def grammar_labels(rules):
    """Label names numbered in order of first appearance (src/main.cpp:84-88)."""
    labels = []
    for r in rules:
        for name in r:
            if name not in labels:
                labels.append(name)
    return labels


def write_grammar(path, rules):
    with open(path, "w") as f:
        f.write("# number of rules\n%d\n# rules\n" % len(rules))
        for r in rules:
            f.write("\t".join(r) + "\n")


def write_graph(path, w: Workload):
    order = np.lexsort((w.lab, w.dst, w.src))
    src, dst, lab = w.src[order], w.dst[order], w.lab[order]
    names = np.array(w.labels, dtype=object)[lab.astype(np.int64) - 1]
    with open(path, "w") as f:
        f.write("# number of edges, number of variables\n%d\t%d\n# edges\n" % (len(src), w.num_vars))
        chunk = 1 << 20
        for s in range(0, len(src), chunk):
            e = min(len(src), s + chunk)
            lines = [f"{a}\t{b}\t{c}" for a, b, c in zip(src[s:e].tolist(), dst[s:e].tolist(), names[s:e].tolist())]
            f.write("\n".join(lines) + "\n")


def _zipf_degrees(rng, n, s, cap, total):
    """Out-degrees ~ Zipf(s) capped at cap (min 1), trimmed/padded at random to
    sum to total (at most n * cap)."""
    total = min(int(total), int(n) * int(cap))
    deg = np.minimum(rng.zipf(s, size=n), cap).astype(np.int64)
    diff = int(total - deg.sum())
    while diff != 0:
        if diff > 0:
            idx = rng.integers(0, n, size=diff)
            np.add.at(deg, idx, 1)
            over = deg > cap
            diff = int(deg[over].sum() - cap * over.sum())
            deg[over] = cap
        else:
            pos = np.nonzero(deg > 1)[0]
            if len(pos) == 0:
                break
            take = rng.choice(pos, size=min(-diff, len(pos)), replace=False)
            deg[take] -= 1
            diff = int(total - deg.sum())
    return deg


def _dedup(src, dst, lab, num_vars):
    key = (src.astype(np.uint64) * np.uint64(num_vars) + dst.astype(np.uint64)) * np.uint64(256) + lab.astype(np.uint64)
    _, idx = np.unique(key, return_index=True)
    keep = np.zeros(len(src), dtype=bool)
    keep[idx] = True
    return keep


def _local_dst(rng, src, num_vars, p_local=0.8, window=256):
    n = len(src)
    local = rng.random(n) < p_local
    off = rng.integers(-window, window + 1, size=n)
    d_local = np.clip(src.astype(np.int64) + off, 0, num_vars - 1)
    d_unif = rng.integers(0, num_vars, size=n)
    return np.where(local, d_local, d_unif).astype(np.uint32)


def _distinct_edges(rng, num_vars, deg, label_of_edge, draw_dst):
    """Edges with the given per-source out-degrees; distinct (src,dst,label) by resampling."""
    src = np.repeat(np.arange(num_vars, dtype=np.uint32), deg)
    lab = label_of_edge(len(src))
    dst = draw_dst(src)
    for _ in range(64):
        keep = _dedup(src, dst, lab, num_vars)
        bad = np.nonzero(~keep)[0]
        if len(bad) == 0:
            break
        dst[bad] = draw_dst(src[bad])
    keep = _dedup(src, dst, lab, num_vars)
    return src[keep], dst[keep], lab[keep]


def dataflow_small(seed=0x5EED0001, num_vars=10_000, num_edges=30_000):
    rng = np.random.default_rng(seed)
    labels = grammar_labels(DATAFLOW_RULES)
    e = labels.index("e") + 1
    deg = _zipf_degrees(rng, num_vars, 2.0, 64, num_edges)
    src, dst, lab = _distinct_edges(rng, num_vars, deg, lambda n: np.full(n, e, np.uint8),
                                    lambda s: _local_dst(rng, s, num_vars))
    return Workload("dataflow_small", num_vars, DATAFLOW_RULES, 0, src, dst, labels, lab,
                    {"seed": seed, "edges_requested": num_edges})


def dataflow_blocks(seed=0x5EED0002, num_blocks=2000, block=1000, num_edges=6_000_000,
                    intra_frac=0.85, exits=10, entries=10, call_window=5, seed_n=True):
    """Block-structured dataflow graph (filter 1); see the module docstring."""
    rng = np.random.default_rng(seed)
    labels = grammar_labels(DATAFLOW_RULES)
    e_id, n_id = labels.index("e") + 1, labels.index("N") + 1
    num_vars = num_blocks * block
    n_intra = int(round(num_edges * intra_frac))
    n_cross = num_edges - n_intra
    # cross edges leave the exits only: at most exits x call_window x entries per block
    max_cross = num_blocks * exits * call_window * entries
    if n_cross > max_cross:
        n_intra += n_cross - max_cross
        n_cross = max_cross
    pos = np.arange(num_vars, dtype=np.int64) % block
    body = np.nonzero(pos < block - exits)[0]          # intra-block sources: all but the exits
    deg = np.zeros(num_vars, dtype=np.int64)
    deg[body] = _zipf_degrees(rng, len(body), 2.0, 64, n_intra)
    blk_start = (np.arange(num_vars, dtype=np.int64) // block) * block

    def draw_intra(s):
        # locality model of dataflow_small, confined to the block body [start, start+block-exits)
        s = s.astype(np.int64)
        lo = blk_start[s]
        hi = lo + (block - exits - 1)
        local = rng.random(len(s)) < 0.8
        d_loc = np.clip(s + rng.integers(-256, 257, size=len(s)), lo, hi)
        d_uni = lo + (rng.random(len(s)) * (hi - lo + 1)).astype(np.int64)
        return np.where(local, d_loc, d_uni).astype(np.uint32)

    s1, d1, l1 = _distinct_edges(rng, num_vars, deg, lambda n: np.full(n, e_id, np.uint8), draw_intra)
    # cross-block edges: block's last `exits` vertices -> first `entries` vertices of one of the next blocks
    exit_v = (np.arange(num_blocks, dtype=np.int64)[:, None] * block + (block - exits) + np.arange(exits)[None, :]).ravel()
    cdeg = np.zeros(num_vars, dtype=np.int64)
    cdeg[exit_v] = _zipf_degrees(rng, len(exit_v), 2.0, call_window * entries, n_cross)

    def draw_cross(s):
        s = s.astype(np.int64)
        b = s // block
        tb = (b + 1 + rng.integers(0, call_window, size=len(s))) % num_blocks
        return (tb * block + rng.integers(0, entries, size=len(s))).astype(np.uint32)

    s2, d2, l2 = _distinct_edges(rng, num_vars, cdeg, lambda n: np.full(n, e_id, np.uint8), draw_cross)
    src = np.concatenate([s1, s2])
    dst = np.concatenate([d1, d2])
    lab = np.concatenate([l1, l2])
    meta = {"seed": seed, "blocks": num_blocks, "block": block, "e_edges": int(len(src)),
            "edges_requested": num_edges, "n_seeded": bool(seed_n)}
    if seed_n:
        src = np.concatenate([src, src])
        dst = np.concatenate([dst, dst])
        lab = np.concatenate([lab, np.full(len(lab), n_id, np.uint8)])
    order = np.lexsort((lab, dst, src))
    return Workload("dataflow_blocks", num_vars, DATAFLOW_RULES, 1, src[order], dst[order], labels, lab[order], meta)


def alias(seed=0x5EED0003, num_vars=1_000_000, num_base_edges=4_000_000, frac_a=0.6, zipf_s=1.8, cap=256,
          p_local=0.8, window=256, block=1000, partner=0, p_cross=0.02):
    """Alias-analysis graph. block=None draws edges over the whole vertex range
    (every vertex then joins one V class and the closure grows as V^2);
    block=B confines each vertex's edges to its B-vertex procedure block.
    partner=P (with block): a fraction p_cross of the edges go instead to the
    partner block P blocks away (blocks b and b + P are partners when b // P is
    even), so procedures call across P-block strides -- with P blocks per
    partition, across partition boundaries -- while the closure stays bounded
    (each call graph component is two blocks)."""
    rng = np.random.default_rng(seed)
    labels = grammar_labels(ALIAS_RULES)
    ids = {n: labels.index(n) + 1 for n in labels}
    deg = _zipf_degrees(rng, num_vars, zipf_s, cap, num_base_edges)
    if block:
        bs = (np.arange(num_vars, dtype=np.int64) // block) * block
        be = np.minimum(bs + block, num_vars) - 1

        nblocks = (num_vars + block - 1) // block

        def draw(s):
            s = s.astype(np.int64)
            lo, hi = bs[s], be[s]
            local = rng.random(len(s)) < p_local
            d_loc = np.clip(s + rng.integers(-window, window + 1, size=len(s)), lo, hi)
            d_uni = lo + (rng.random(len(s)) * (hi - lo + 1)).astype(np.int64)
            d = np.where(local, d_loc, d_uni)
            if partner:
                b = s // block
                pb = np.where((b // partner) % 2 == 0, b + partner, b - partner)
                cross = (rng.random(len(s)) < p_cross) & (pb >= 0) & (pb < nblocks)
                off = d - lo
                d = np.where(cross, np.minimum(pb * block + off, num_vars - 1), d)
            return d.astype(np.uint32)
    else:
        def draw(s):
            return _local_dst(rng, s, num_vars, p_local, window)

    def lab_of(n):
        return np.where(rng.random(n) < frac_a, ids["a"], ids["d"]).astype(np.uint8)

    src, dst, lab = _distinct_edges(rng, num_vars, deg, lab_of, draw)
    inv = np.where(lab == ids["a"], ids["a_bar"], ids["d_bar"]).astype(np.uint8)
    s_all = np.concatenate([src, dst])
    d_all = np.concatenate([dst, src])
    l_all = np.concatenate([lab, inv])
    keep = _dedup(s_all, d_all, l_all, num_vars)
    s_all, d_all, l_all = s_all[keep], d_all[keep], l_all[keep]
    order = np.lexsort((l_all, d_all, s_all))
    return Workload("alias", num_vars, ALIAS_RULES, 0, s_all[order], d_all[order], labels, l_all[order],
                    {"seed": seed, "base_edges": int(len(src)), "block": block, "partner": partner,
                     "p_cross": p_cross if partner else 0.0})


POINTSTO_RULES = [("M", "DV", "d"), ("DV", "-d", "V"), ("V", "MAM", "AMs"), ("MAM", "MAs", "Mq"), ("Mq",),
                  ("Mq", "M"), ("MAs",), ("MAs", "MAs", "MA"), ("MA", "Mq", "-a"), ("AMs",), ("AMs", "AMs", "AM"),
                  ("AM", "a", "Mq")]


def pointsto(seed=0x5EED0004, num_vars=2000, num_edges=8000, frac_a=0.4):
    """Points-to grammar with epsilon, unary and binary rules (the reference's
    sample grammar); a/d edges plus their -a/-d inverses, locality as dataflow_small."""
    rng = np.random.default_rng(seed)
    labels = grammar_labels(POINTSTO_RULES)
    ids = {n: labels.index(n) + 1 for n in labels}
    deg = _zipf_degrees(rng, num_vars, 2.0, 64, num_edges)

    def lab_of(n):
        return np.where(rng.random(n) < frac_a, ids["a"], ids["d"]).astype(np.uint8)

    src, dst, lab = _distinct_edges(rng, num_vars, deg, lab_of, lambda s: _local_dst(rng, s, num_vars, 0.8, 64))
    inv = np.where(lab == ids["a"], ids["-a"], ids["-d"]).astype(np.uint8)
    s_all = np.concatenate([src, dst])
    d_all = np.concatenate([dst, src])
    l_all = np.concatenate([lab, inv])
    keep = _dedup(s_all, d_all, l_all, num_vars)
    s_all, d_all, l_all = s_all[keep], d_all[keep], l_all[keep]
    order = np.lexsort((l_all, d_all, s_all))
    return Workload("pointsto", num_vars, POINTSTO_RULES, 0, s_all[order], d_all[order], labels, l_all[order],
                    {"seed": seed})


def random_grammar_graph(seed, num_vars, num_edges, num_labels, num_rules, eps=True, unary=True):
    """Small random normalised grammar + graph (parity-test fuzzing)."""
    rng = np.random.default_rng(seed)
    names = [f"L{i}" for i in range(num_labels)]
    rules = []
    for _ in range(num_rules):
        kind = rng.integers(0, 10)
        lhs = names[rng.integers(0, num_labels)]
        if kind == 0 and eps:
            rules.append((lhs,))
        elif kind <= 2 and unary:
            rules.append((lhs, names[rng.integers(0, num_labels)]))
        else:
            rules.append((lhs, names[rng.integers(0, num_labels)], names[rng.integers(0, num_labels)]))
    labels = grammar_labels(rules)
    # graph labels: any label that appears in the grammar
    src = rng.integers(0, num_vars, size=num_edges).astype(np.uint32)
    dst = _local_dst(rng, src, num_vars, 0.7, 64)
    lab = rng.integers(1, len(labels) + 1, size=num_edges).astype(np.uint8)
    keep = _dedup(src, dst, lab, num_vars)
    src, dst, lab = src[keep], dst[keep], lab[keep]
    order = np.lexsort((lab, dst, src))
    return Workload(f"random{seed}", num_vars, rules, 0, src[order], dst[order], labels, lab[order], {"seed": seed})


def batch_mix(seed=0x5EED0005, jobs=512, vmin=1_000, vmax=200_000, rate=200.0):
    """Mix of independent jobs: log-uniform sizes, half dataflow / half alias, Poisson arrivals."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for j in range(jobs):
        v = int(np.exp(rng.uniform(np.log(vmin), np.log(vmax))))
        m = float(rng.uniform(3, 5))
        t += float(rng.exponential(1.0 / rate))
        kind = "dataflow" if j % 2 == 0 else "alias"
        out.append({"job": j, "kind": kind, "num_vars": v, "edges": int(m * v), "arrival_s": t,
                    "seed": int(rng.integers(0, 2**63 - 1))})
    return out
