"""CPU tests of the compressed edge stream (the reference's COMPRESSED=1 spill
format, src/main.cpp:510-596): the oracle's writer against an independent
numpy packing of its sorted edge list, and the stream's own invariants."""
import numpy as np
import pytest

import grg_gen as G


def pack_csr5(src, dst, lab, v_begin, v_end):
    """Edges of source rows [v_begin, v_end) ordered by (source, label,
    destination), 5 bytes each (little-endian destination, label), plus the
    per-row edge counts."""
    src = np.asarray(src, np.int64)
    sel = (src >= v_begin) & (src < v_end)
    s, d, l = src[sel], np.asarray(dst, np.uint32)[sel], np.asarray(lab, np.uint8)[sel]
    order = np.lexsort((d, l, s))
    s, d, l = s[order], d[order], l[order]
    out = np.zeros((len(s), 5), np.uint8)
    out[:, :4] = d.astype("<u4").view(np.uint8).reshape(-1, 4)
    out[:, 4] = l
    deg = np.bincount(s - v_begin, minlength=v_end - v_begin).astype(np.uint32)
    return out.reshape(-1), deg


def unpack_csr5(stream, deg, v_begin):
    rec = np.asarray(stream, np.uint8).reshape(-1, 5)
    dst = rec[:, :4].copy().view("<u4").reshape(-1)
    lab = rec[:, 4].copy()
    src = np.repeat(np.arange(v_begin, v_begin + len(deg), dtype=np.uint32), deg)
    return src, dst, lab


WORKLOADS = [
    lambda: G.pointsto(seed=31, num_vars=700, num_edges=2000),
    lambda: G.dataflow_small(seed=32, num_vars=1500, num_edges=4500),
    lambda: G.alias(seed=33, num_vars=2000, num_base_edges=5000, block=500),
]


@pytest.mark.parametrize("make", WORKLOADS)
def test_oracle_stream_matches_numpy_packing(oracle_mod, make):
    w = make()
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    s, d, l = r.edges()
    for lo, hi in [(0, w.num_vars), (0, 1), (w.num_vars // 3, w.num_vars // 2), (5, 5)]:
        got, deg = r.csr5(lo, hi)
        want, wdeg = pack_csr5(s, d, l, lo, hi)
        assert np.array_equal(got, want), (lo, hi)
        assert np.array_equal(deg, wdeg), (lo, hi)
        assert int(deg.sum()) * 5 == len(got)


def test_stream_round_trips_through_unpack(oracle_mod):
    w = G.pointsto(seed=34, num_vars=500, num_edges=1500)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, w.src, w.dst, w.lab)
    stream, deg = r.csr5()
    src, dst, lab = unpack_csr5(stream, deg, 0)
    # re-closing the closed edge set adds nothing
    r2 = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 0, src, dst, lab)
    assert [int(x) for x in r2.label_counts()] == [int(x) for x in r.label_counts()]
    assert r2.set_hash == r.set_hash
    # rows ascending, then labels, then destinations: the packed key strictly increases
    key = (src.astype(np.uint64) << np.uint64(40)) | (lab.astype(np.uint64) << np.uint64(32)) | dst
    assert np.all(np.diff(key.astype(np.int64)) > 0)


def test_degree_matches_oracle_degree(oracle_mod):
    w = G.dataflow_small(seed=35, num_vars=800, num_edges=2400)
    r = oracle_mod.closure(w.num_vars, w.rule_ids(), w.num_labels, 1, w.src, w.dst, w.lab)
    _, deg = r.csr5()
    edges, _ = r.degree()
    assert np.array_equal(deg, edges)
