"""Independent pure-Python CFL-reachability fixpoint (small cases only).

Test infrastructure: an edge-at-a-time worklist algorithm (the textbook
dynamic-transitive-closure formulation of CFL reachability), written
independently of the round-based C oracle so the two can be cross-checked.

Semantics follow the reference (src/kernel.cu): epsilon rules add (v,v,A)
for every vertex, unary rules A ::= B copy edges, binary rules A ::= B C join
B(i,k) with C(k,j). filter_flag 1 drops every unary rule; it is only exact
(and only accepted here) when no binary rule's second symbol is derivable.
"""
from collections import defaultdict, deque


def closure(num_vars, rules, edges, filter_flag=0):
    """rules: iterable of (lhs, rhs1, rhs2) label ids (0 = absent).
    edges: iterable of (src, dst, label). Returns a set of (src, dst, label)."""
    rules = [tuple(int(x) for x in r) for r in rules]
    active = [r for r in rules if not (filter_flag and r[1] and not r[2])]
    derivable = {r[0] for r in active}
    if filter_flag and any(r[1] and r[2] and r[2] in derivable for r in active):
        raise ValueError("filter_flag=1 is schedule-dependent for this grammar")
    unary = defaultdict(list)       # B -> [A]
    by_first = defaultdict(list)    # B -> [(A, C)]
    by_second = defaultdict(list)   # C -> [(A, B)]
    for a, b, c in active:
        if b and c:
            by_first[b].append((a, c))
            by_second[c].append((a, b))
        elif b:
            unary[b].append(a)
    out = defaultdict(set)          # (label, src) -> {dst}
    inn = defaultdict(set)          # (label, dst) -> {src}
    known = set()
    work = deque()

    def add(s, d, l):
        if (s, d, l) in known:
            return
        known.add((s, d, l))
        out[(l, s)].add(d)
        inn[(l, d)].add(s)
        work.append((s, d, l))

    for s, d, l in edges:
        add(int(s), int(d), int(l))
    for a, b, c in active:
        if b == 0:
            for v in range(num_vars):
                add(v, v, a)
    while work:
        i, k, lb = work.popleft()
        for a in unary[lb]:
            add(i, k, a)
        for a, c in by_first[lb]:          # lb(i,k) . c(k,j)
            for j in list(out[(c, k)]):
                add(i, j, a)
        for a, b in by_second[lb]:         # b(h,i) . lb(i,k)
            for h in list(inn[(b, i)]):
                add(h, k, a)
    return known
