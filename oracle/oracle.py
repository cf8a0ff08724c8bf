"""ctypes wrapper of the CPU oracle (oracle/grg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py`` as the checker. The product path
(the CUDA library and its host code) never imports it.

Parity status: UNPINNED against reference output (the reference has no tests,
golden vectors or CPU closure code and cannot run without a GPU and boost);
the oracle is cross-checked against an independent pure-Python worklist
fixpoint in ``tests/naive_cfl.py``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgrg_oracle.so")

ORC_OK = 0
ORC_E_ARG = -1
ORC_E_FILTER = -2
ORC_E_NOMEM = -3
ORC_E_IO = -4
ORC_E_LABEL = -5
ORC_E_RANGE = -6
MAX_RULES = 64
MAX_LABELS = 126
NAME_LEN = 64
NSTAT = 8
# round statistics columns
STAT_NAMES = ("new_edges", "new_elems", "left_elems", "right_elems",
              "oldleft_left_elems", "oldleft_right_elems", "unary_elems", "cand_elems")

_lib = None


def build(quiet: bool = True) -> str:
    """Compile the oracle shared library with the committed Makefile."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.oracle_parse_grammar.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), P,
                                           ctypes.POINTER(ctypes.c_int), P]
        L.oracle_parse_graph_header.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64),
                                                ctypes.POINTER(ctypes.c_uint32)]
        L.oracle_parse_graph.argtypes = [ctypes.c_char_p, ctypes.c_int, P, ctypes.c_uint64, ctypes.c_uint32,
                                         P, P, P]
        L.oracle_closure.restype = P
        L.oracle_closure.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_int, P, ctypes.c_int,
                                     ctypes.c_uint64, P, P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.oracle_total.restype = ctypes.c_uint64
        L.oracle_total.argtypes = [P]
        L.oracle_set_hash.restype = ctypes.c_uint64
        L.oracle_set_hash.argtypes = [P]
        L.oracle_num_rounds.restype = ctypes.c_uint32
        L.oracle_num_rounds.argtypes = [P]
        L.oracle_label_counts.argtypes = [P, P]
        L.oracle_round_stats.argtypes = [P, P]
        L.oracle_degree.argtypes = [P, P, P]
        L.oracle_export.restype = ctypes.c_uint64
        L.oracle_export.argtypes = [P, P, P, P, ctypes.c_uint64]
        L.oracle_export_csr5.restype = ctypes.c_uint64
        L.oracle_export_csr5.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, P, P, ctypes.c_uint64]
        L.oracle_free.argtypes = [P]
        L.oracle_edge_hash.restype = ctypes.c_uint64
        L.oracle_edge_hash.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


@dataclass
class Grammar:
    rules: np.ndarray          # int32 [num_rules, 3], label ids 1-based, 0 = absent
    labels: list               # label names; id = index + 1

    @property
    def num_labels(self) -> int:
        return len(self.labels)

    def label_id(self, name: str) -> int:
        return self.labels.index(name) + 1


def parse_grammar(path: str) -> Grammar:
    nr = ctypes.c_int()
    nl = ctypes.c_int()
    rules = np.zeros(3 * MAX_RULES, dtype=np.int32)
    names = ctypes.create_string_buffer(MAX_LABELS * NAME_LEN)
    rc = lib().oracle_parse_grammar(path.encode(), ctypes.byref(nr), _ptr(rules), ctypes.byref(nl), names)
    if rc != ORC_OK:
        raise ValueError(f"oracle grammar parse failed ({rc}) for {path}")
    raw = names.raw
    labels = [raw[i * NAME_LEN:(i + 1) * NAME_LEN].split(b"\0", 1)[0].decode() for i in range(nl.value)]
    return Grammar(rules[:3 * nr.value].reshape(-1, 3).copy(), labels)


def parse_graph(path: str, g: Grammar):
    ne = ctypes.c_uint64()
    nv = ctypes.c_uint32()
    rc = lib().oracle_parse_graph_header(path.encode(), ctypes.byref(ne), ctypes.byref(nv))
    if rc != ORC_OK:
        raise ValueError(f"oracle graph header parse failed ({rc})")
    n = ne.value
    src = np.zeros(n, dtype=np.uint32)
    dst = np.zeros(n, dtype=np.uint32)
    lab = np.zeros(n, dtype=np.uint8)
    names = ctypes.create_string_buffer(MAX_LABELS * NAME_LEN)
    for i, s in enumerate(g.labels):
        b = s.encode()
        ctypes.memmove(ctypes.addressof(names) + i * NAME_LEN, b, len(b))
    rc = lib().oracle_parse_graph(path.encode(), g.num_labels, names, n, nv.value, _ptr(src), _ptr(dst), _ptr(lab))
    if rc != ORC_OK:
        raise ValueError(f"oracle graph parse failed ({rc})")
    return nv.value, src, dst, lab


class ClosureResult:
    def __init__(self, handle, num_labels, num_vars):
        self._h = handle
        self.num_labels = num_labels
        self.num_vars = num_vars

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_free(self._h)
            self._h = None

    @property
    def total(self) -> int:
        return int(lib().oracle_total(self._h))

    @property
    def set_hash(self) -> int:
        return int(lib().oracle_set_hash(self._h))

    @property
    def rounds(self) -> int:
        return int(lib().oracle_num_rounds(self._h))

    def label_counts(self) -> np.ndarray:
        out = np.zeros(self.num_labels, dtype=np.uint64)
        lib().oracle_label_counts(self._h, _ptr(out))
        return out

    def round_stats(self) -> np.ndarray:
        out = np.zeros((self.rounds, NSTAT), dtype=np.uint64)
        lib().oracle_round_stats(self._h, _ptr(out))
        return out

    def degree(self):
        e = np.zeros(self.num_vars, dtype=np.uint32)
        el = np.zeros(self.num_vars, dtype=np.uint32)
        lib().oracle_degree(self._h, _ptr(e), _ptr(el))
        return e, el

    def edges(self):
        """Closure edges sorted by (label, src, dst)."""
        n = int(lib().oracle_export(self._h, None, None, None, 0))
        src = np.zeros(n, dtype=np.uint32)
        dst = np.zeros(n, dtype=np.uint32)
        lab = np.zeros(n, dtype=np.uint8)
        lib().oracle_export(self._h, _ptr(src), _ptr(dst), _ptr(lab), n)
        return src, dst, lab

    def csr5(self, v_begin: int = 0, v_end: int | None = None):
        """Rows [v_begin, v_end) in the compressed spill format: (uint8 stream of
        5 bytes per edge, uint32 edge count per vertex)."""
        if v_end is None:
            v_end = self.num_vars
        deg = np.zeros(max(v_end - v_begin, 0), dtype=np.uint32)
        n = int(lib().oracle_export_csr5(self._h, v_begin, v_end, None, _ptr(deg), 0))
        out = np.zeros(n * 5, dtype=np.uint8)
        lib().oracle_export_csr5(self._h, v_begin, v_end, _ptr(out), _ptr(deg), n)
        return out, deg


class OracleError(RuntimeError):
    def __init__(self, code):
        super().__init__(f"oracle closure failed with status {code}")
        self.code = code


def closure(num_vars, rules, num_labels, filter_flag, src, dst, lab, row_mask=None, nthreads=None):
    rules = np.ascontiguousarray(np.asarray(rules, dtype=np.int32).reshape(-1))
    src = np.ascontiguousarray(src, dtype=np.uint32)
    dst = np.ascontiguousarray(dst, dtype=np.uint32)
    lab = np.ascontiguousarray(lab, dtype=np.uint8)
    if row_mask is not None:
        row_mask = np.ascontiguousarray(row_mask, dtype=np.uint8)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    st = ctypes.c_int()
    h = lib().oracle_closure(num_vars, num_labels, len(rules) // 3, _ptr(rules), filter_flag,
                             len(src), _ptr(src), _ptr(dst), _ptr(lab), _ptr(row_mask), nthreads,
                             ctypes.byref(st))
    if not h:
        raise OracleError(st.value)
    return ClosureResult(h, num_labels, num_vars)


def edge_hash(label: int, src: int, dst: int) -> int:
    return int(lib().oracle_edge_hash(label, src, dst))
