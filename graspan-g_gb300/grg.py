"""Python host interface of the GB300 closure engine (ctypes over libgrg.so).

Mirrors the reference's host<->CUDA interface (src/kernel.h:115-129) through
the C ABI declared in include/grg.h. There is no CPU fallback: if the CUDA
library is missing, ``load_library`` raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("GRG_LIB") or os.path.join(HERE, "_build", "libgrg.so")
COMP_PATH = os.path.join(HERE, "_build", "comp")

OK = 0
NEED_REPARTITION = 1
PAUSED = 2
E_ARG, E_CUDA, E_NOMEM, E_FILTER, E_IO, E_LABEL, E_RANGE, E_STATE, E_NODEV, E_INTERNAL = -1, -2, -3, -4, -5, -6, -7, -8, -9, -10
MAX_RULES = 64
MAX_LABELS = 63
NAME_LEN = 64

# every entry point declared in include/grg.h
EXPORTS = (
    "grg_error_string", "grg_last_error", "grg_create", "grg_destroy", "grg_device", "grg_set_stream",
    "grg_set_kernel_timing", "grg_transfer_rules", "grg_allocate_pool", "grg_load_edges", "grg_closure",
    "grg_label_counts", "grg_get_degree", "grg_set_hash", "grg_export_edges", "grg_parse_grammar",
    "grg_parse_graph_header", "grg_parse_graph", "grg_closure_noalloc", "grg_batch_begin", "grg_batch_admit",
    "grg_batch_step", "grg_batch_result", "grg_batch_release", "grg_get_rules", "grg_closure_ex",
    "grg_load_elements", "grg_export_elements", "grg_range_counts", "grg_set_pool_limit", "grg_part_create",
    "grg_part_destroy", "grg_part_load_edges", "grg_part_run", "grg_part_label_counts", "grg_part_bounds",
    "grg_set_device_rounds", "grg_range_reach", "grg_set_join_window", "grg_export_csr5", "grg_load_csr5",
    "grg_part_export_csr5", "grg_part_save", "grg_part_restore", "grg_part_set_checkpoint", "grg_part_set_run_budget",
    "grg_set_layout", "grg_set_push", "grg_set_join_items",
)


class GrgError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"grg status {status}: {msg}")
        self.status = status


class Stats(ctypes.Structure):
    _fields_ = [
        ("total_edges", ctypes.c_uint64), ("rounds", ctypes.c_uint64), ("delta_elems", ctypes.c_uint64),
        ("left_elems", ctypes.c_uint64), ("right_elems", ctypes.c_uint64), ("out_elems", ctypes.c_uint64),
        ("retry_records", ctypes.c_uint64), ("grow_rows", ctypes.c_uint64), ("pool_elems_used", ctypes.c_uint64),
        ("pool_elems_cap", ctypes.c_uint64), ("closure_ms", ctypes.c_double), ("join_ms", ctypes.c_double),
        ("join_launches", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
        ("join_phase_cycles", ctypes.c_uint64 * 5), ("window_out_elems", ctypes.c_uint64),
        ("wide_window", ctypes.c_uint64), ("gather_ms", ctypes.c_double),
        ("window_tuned", ctypes.c_uint64), ("window_trial_ms", ctypes.c_double * 2),
        ("column_labels", ctypes.c_uint64), ("push_flat", ctypes.c_uint64), ("push_tuned", ctypes.c_uint64),
        ("push_trial_ms", ctypes.c_double * 2), ("join_elements", ctypes.c_uint64),
        ("items_trial_ms", ctypes.c_double * 2), ("window_noslot_items", ctypes.c_uint64),
        ("candidates", ctypes.c_uint64), ("join_inserts", ctypes.c_uint64), ("direct_inserts", ctypes.c_uint64),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["join_phase_cycles"] = list(d["join_phase_cycles"])
        d["window_trial_ms"] = list(d["window_trial_ms"])
        d["push_trial_ms"] = list(d["push_trial_ms"])
        d["items_trial_ms"] = list(d["items_trial_ms"])
        return d


class PartStats(ctypes.Structure):
    _fields_ = [
        ("total_edges", ctypes.c_uint64), ("num_parts", ctypes.c_uint32), ("schedule", ctypes.c_uint32),
        ("supersteps", ctypes.c_uint64), ("runs", ctypes.c_uint64), ("skipped", ctypes.c_uint64),
        ("splits", ctypes.c_uint64), ("rounds", ctypes.c_uint64), ("h2d_bytes", ctypes.c_uint64),
        ("d2h_bytes", ctypes.c_uint64), ("ms", ctypes.c_double), ("stage_ms", ctypes.c_double),
        ("load_ms", ctypes.c_double), ("closure_ms", ctypes.c_double), ("export_ms", ctypes.c_double),
        ("count_ms", ctypes.c_double), ("prefetched", ctypes.c_uint64), ("prefetch_hits", ctypes.c_uint64),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["schedule"] = ("stream", "pairs")[d["schedule"]]
        return d


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libgrg.so (fails loudly when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise GrgError(E_STATE, f"CUDA library {path} is missing; run graspan-g_gb300/build.py")
    L = ctypes.CDLL(path)
    P, I, U32, U64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64
    L.grg_error_string.restype = ctypes.c_char_p
    L.grg_error_string.argtypes = [I]
    L.grg_last_error.restype = ctypes.c_char_p
    L.grg_last_error.argtypes = [P]
    L.grg_create.argtypes = [ctypes.POINTER(P), I]
    L.grg_destroy.argtypes = [P]
    L.grg_destroy.restype = None
    L.grg_device.argtypes = [P]
    L.grg_set_stream.argtypes = [P, P]
    L.grg_set_kernel_timing.argtypes = [P, I]
    L.grg_set_device_rounds.argtypes = [P, I]
    L.grg_set_join_window.argtypes = [P, I]
    L.grg_set_layout.argtypes = [P, I]
    L.grg_set_push.argtypes = [P, I]
    L.grg_set_join_items.argtypes = [P, I]
    L.grg_transfer_rules.argtypes = [P, I, P, I]
    L.grg_allocate_pool.argtypes = [P, U64]
    L.grg_load_edges.argtypes = [P, U32, U64, P, P, P, I]
    L.grg_closure.argtypes = [P, U32, ctypes.POINTER(Stats)]
    L.grg_label_counts.argtypes = [P, P]
    L.grg_get_degree.argtypes = [P, U32, U32, P]
    L.grg_set_hash.argtypes = [P, ctypes.POINTER(U64)]
    L.grg_export_edges.argtypes = [P, U64, P, P, P, ctypes.POINTER(U64)]
    L.grg_parse_grammar.argtypes = [ctypes.c_char_p, ctypes.POINTER(I), P, ctypes.POINTER(I), P]
    L.grg_parse_graph_header.argtypes = [ctypes.c_char_p, ctypes.POINTER(U64), ctypes.POINTER(U32)]
    L.grg_parse_graph.argtypes = [ctypes.c_char_p, I, P, U64, U32, P, P, P]
    L.grg_closure_noalloc.argtypes = [I, P, I, P, I, U32, U32, U64, P, P, P, P, P, ctypes.POINTER(U64)]
    L.grg_batch_begin.argtypes = [P, U32, U32, I, P, I, U32]
    L.grg_batch_admit.argtypes = [P, U32, U32, U32, U64, P, P, P, I, U64]
    L.grg_batch_step.argtypes = [P, U32, P, ctypes.POINTER(U64)]
    L.grg_batch_result.argtypes = [P, U32, U32, U32, P, ctypes.POINTER(U64)]
    L.grg_batch_release.argtypes = [P, U32]
    L.grg_get_rules.argtypes = [P, ctypes.POINTER(I), P, ctypes.POINTER(I)]
    L.grg_closure_ex.argtypes = [P, U32, U32, ctypes.POINTER(Stats)]
    L.grg_load_elements.argtypes = [P, U32, U64, P, P, U32, I]
    L.grg_export_elements.argtypes = [P, U32, U32, U64, P, P, ctypes.POINTER(U64)]
    L.grg_range_counts.argtypes = [P, U32, U32, P, ctypes.POINTER(U64)]
    L.grg_set_pool_limit.argtypes = [P, U64]
    L.grg_range_reach.argtypes = [P, U32, U32, U64, U32, P, P]
    L.grg_export_csr5.argtypes = [P, U32, U32, U64, P, P, ctypes.POINTER(U64)]
    L.grg_load_csr5.argtypes = [P, U32, U32, U32, P, U64, P, ctypes.c_int]
    L.grg_part_create.argtypes = [ctypes.POINTER(P), P, U32, U32]
    L.grg_part_destroy.argtypes = [P]
    L.grg_part_destroy.restype = None
    L.grg_part_load_edges.argtypes = [P, U64, P, P, P]
    L.grg_part_run.argtypes = [P, U32, ctypes.POINTER(PartStats)]
    L.grg_part_label_counts.argtypes = [P, P, ctypes.POINTER(U64)]
    L.grg_part_bounds.argtypes = [P, U32, P, ctypes.POINTER(U32)]
    L.grg_part_export_csr5.argtypes = [P, U32, U64, P, P, ctypes.POINTER(U64)]
    L.grg_part_save.argtypes = [P, ctypes.c_char_p]
    L.grg_part_restore.argtypes = [ctypes.POINTER(P), P, ctypes.c_char_p]
    L.grg_part_set_checkpoint.argtypes = [P, ctypes.c_char_p, U32]
    L.grg_part_set_run_budget.argtypes = [P, U64]
    _lib = L
    return L


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def error_string(status: int) -> str:
    return load_library().grg_error_string(status).decode()


@dataclass
class Grammar:
    rules: np.ndarray     # int32 [num_rules, 3]
    labels: list

    @property
    def num_labels(self):
        return len(self.labels)


def parse_grammar(path: str) -> Grammar:
    L = load_library()
    nr, nl = ctypes.c_int(), ctypes.c_int()
    rules = np.zeros(3 * MAX_RULES, dtype=np.int32)
    names = ctypes.create_string_buffer(MAX_LABELS * NAME_LEN)
    st = L.grg_parse_grammar(path.encode(), ctypes.byref(nr), _ptr(rules), ctypes.byref(nl), names)
    if st != OK:
        raise GrgError(st, f"parse_grammar({path}): {error_string(st)}")
    raw = names.raw
    labels = [raw[i * NAME_LEN:(i + 1) * NAME_LEN].split(b"\0", 1)[0].decode() for i in range(nl.value)]
    return Grammar(rules[:3 * nr.value].reshape(-1, 3).copy(), labels)


def _names_buffer(labels):
    names = ctypes.create_string_buffer(MAX_LABELS * NAME_LEN)
    for i, s in enumerate(labels):
        b = s.encode()
        ctypes.memmove(ctypes.addressof(names) + i * NAME_LEN, b, len(b))
    return names


def parse_graph(path: str, g: Grammar):
    L = load_library()
    ne, nv = ctypes.c_uint64(), ctypes.c_uint32()
    st = L.grg_parse_graph_header(path.encode(), ctypes.byref(ne), ctypes.byref(nv))
    if st != OK:
        raise GrgError(st, f"parse_graph_header({path})")
    n = ne.value
    src = np.zeros(n, np.uint32)
    dst = np.zeros(n, np.uint32)
    lab = np.zeros(n, np.uint8)
    st = L.grg_parse_graph(path.encode(), g.num_labels, _names_buffer(g.labels), n, nv.value,
                           _ptr(src), _ptr(dst), _ptr(lab))
    if st != OK:
        raise GrgError(st, f"parse_graph({path}): {error_string(st)}")
    return nv.value, src, dst, lab


class Context:
    """One closure engine context on one GPU."""

    def __init__(self, device: int = 0):
        self._L = load_library()
        h = ctypes.c_void_p()
        st = self._L.grg_create(ctypes.byref(h), device)
        if st != OK:
            raise GrgError(st, f"grg_create: {error_string(st)}")
        self._h = h
        self.num_labels = 0
        self.num_vars = 0

    def close(self):
        if getattr(self, "_h", None):
            self._L.grg_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st != OK:
            msg = self._L.grg_last_error(self._h).decode() if self._h else ""
            raise GrgError(st, f"{what}: {error_string(st)} {msg}")

    @property
    def device(self) -> int:
        return self._L.grg_device(self._h)

    def set_stream(self, stream_handle: int | None):
        self._check(self._L.grg_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)), "set_stream")

    def set_kernel_timing(self, on: bool):
        self._check(self._L.grg_set_kernel_timing(self._h, int(bool(on))), "set_kernel_timing")

    def set_join_window(self, mode: int):
        """0 = narrow (8 elements), 1 = wide (12), 2 = tuned per degree key (the
        default), 3 = tuned and measured again even when the key is cached."""
        self._check(self._L.grg_set_join_window(self._h, mode), "set_join_window")

    def set_join_items(self, mode: int):
        """Right-hand items of CSR-copied labels: 0 ids, 1 table elements, 2 tuned
        with the window (default), 3 tuned and measured again."""
        self._check(self._L.grg_set_join_items(self._h, mode), "set_join_items")

    def set_push(self, mode: int):
        """Push kernel: 0 one lane per record, 1 edges dealt over the lanes, 2 tuned
        per degree key (default), 3 tuned and measured again."""
        self._check(self._L.grg_set_push(self._h, mode), "set_push")

    def set_layout(self, mode: int):
        """0 (default): every label stored by source; 1: labels the grammar allows
        stored by destination (pushed joins). Takes effect at the next load."""
        self._check(self._L.grg_set_layout(self._h, mode), "set_layout")

    def set_device_rounds(self, on: bool):
        self._check(self._L.grg_set_device_rounds(self._h, int(bool(on))), "set_device_rounds")

    def transfer_rules(self, rules, num_labels: int):
        r = np.ascontiguousarray(np.asarray(rules, dtype=np.int32).reshape(-1))
        self._check(self._L.grg_transfer_rules(self._h, len(r) // 3, _ptr(r), num_labels), "transfer_rules")
        self.num_labels = num_labels

    def allocate_pool(self, pool_bytes: int = 0):
        self._check(self._L.grg_allocate_pool(self._h, pool_bytes), "allocate_pool")

    def load_edges(self, num_vars, src, dst, lab):
        """Host numpy arrays (copied to the device)."""
        src = np.ascontiguousarray(src, dtype=np.uint32)
        dst = np.ascontiguousarray(dst, dtype=np.uint32)
        lab = np.ascontiguousarray(lab, dtype=np.uint8)
        self._check(self._L.grg_load_edges(self._h, num_vars, len(src), _ptr(src), _ptr(dst), _ptr(lab), 0),
                    "load_edges")
        self.num_vars = num_vars

    def load_edges_device(self, num_vars, num_edges, src_ptr: int, dst_ptr: int, lab_ptr: int):
        """Device pointers (e.g. torch tensors' data_ptr())."""
        self._check(self._L.grg_load_edges(self._h, num_vars, num_edges, ctypes.c_void_p(src_ptr),
                                           ctypes.c_void_p(dst_ptr), ctypes.c_void_p(lab_ptr), 1),
                    "load_edges_device")
        self.num_vars = num_vars

    def closure(self, filter_flag: int) -> dict:
        s = Stats()
        self._check(self._L.grg_closure(self._h, filter_flag, ctypes.byref(s)), "closure")
        return s.as_dict()

    def label_counts(self) -> np.ndarray:
        out = np.zeros(self.num_labels, dtype=np.uint64)
        self._check(self._L.grg_label_counts(self._h, _ptr(out)), "label_counts")
        return out

    def set_hash(self) -> int:
        h = ctypes.c_uint64()
        self._check(self._L.grg_set_hash(self._h, ctypes.byref(h)), "set_hash")
        return h.value

    def degree(self, first_var=0, last_var=None):
        if last_var is None:
            last_var = self.num_vars - 1
        n = last_var - first_var + 1
        out = np.zeros(6 * n, dtype=np.uint32)
        self._check(self._L.grg_get_degree(self._h, first_var, last_var, _ptr(out)), "get_degree")
        return out.reshape(6, n)

    def export_edges(self):
        n = ctypes.c_uint64()
        self._check(self._L.grg_export_edges(self._h, 0, None, None, None, ctypes.byref(n)), "export_edges")
        m = n.value
        src = np.zeros(m, np.uint32)
        dst = np.zeros(m, np.uint32)
        lab = np.zeros(m, np.uint8)
        self._check(self._L.grg_export_edges(self._h, m, _ptr(src), _ptr(dst), _ptr(lab), ctypes.byref(n)),
                    "export_edges")
        order = np.lexsort((dst, src, lab))
        return src[order], dst[order], lab[order]

    # ---- element images (out-of-core partitions)
    def set_pool_limit(self, pool_bytes: int):
        self._check(self._L.grg_set_pool_limit(self._h, pool_bytes), "set_pool_limit")

    def load_elements(self, num_vars, recs, stamps, mark_after=0):
        """recs: uint32 [n, 8] element records; stamps: uint32 [n]."""
        recs = np.ascontiguousarray(recs, dtype=np.uint32).reshape(-1, 8)
        stamps = np.ascontiguousarray(stamps, dtype=np.uint32)
        self._check(self._L.grg_load_elements(self._h, num_vars, len(stamps), _ptr(recs), _ptr(stamps), mark_after, 0),
                    "load_elements")
        self.num_vars = num_vars

    def closure_ex(self, filter_flag: int, run_stamp: int) -> dict:
        s = Stats()
        self._check(self._L.grg_closure_ex(self._h, filter_flag, run_stamp, ctypes.byref(s)), "closure_ex")
        return s.as_dict()

    def export_elements(self, v_begin=0, v_end=None):
        if v_end is None:
            v_end = self.num_vars
        n = ctypes.c_uint64()
        st = self._L.grg_export_elements(self._h, v_begin, v_end, 0, None, None, ctypes.byref(n))
        if st not in (OK, E_RANGE):
            self._check(st, "export_elements")
        recs = np.zeros((n.value, 8), np.uint32)
        stamps = np.zeros(n.value, np.uint32)
        self._check(self._L.grg_export_elements(self._h, v_begin, v_end, n.value, _ptr(recs), _ptr(stamps),
                                                ctypes.byref(n)), "export_elements")
        return recs, stamps

    def export_csr5(self, v_begin=0, v_end=None):
        """Rows [v_begin, v_end) as the compressed edge stream: (uint8 array of
        5 bytes per edge, uint32 edges per source vertex)."""
        if v_end is None:
            v_end = self.num_vars
        n = ctypes.c_uint64()
        st = self._L.grg_export_csr5(self._h, v_begin, v_end, 0, None, None, ctypes.byref(n))
        if st not in (OK, E_RANGE):
            self._check(st, "export_csr5")
        out = np.zeros(n.value * 5, np.uint8)
        deg = np.zeros(v_end - v_begin, np.uint32)
        self._check(self._L.grg_export_csr5(self._h, v_begin, v_end, n.value, _ptr(out), _ptr(deg),
                                            ctypes.byref(n)), "export_csr5")
        return out, deg

    def load_csr5(self, num_vars, stream, degree, v_begin=0):
        """Load a graph from a compressed edge stream whose rows start at v_begin."""
        stream = np.ascontiguousarray(stream, dtype=np.uint8)
        degree = np.ascontiguousarray(degree, dtype=np.uint32)
        if stream.size % 5:
            raise ValueError("stream length is not a multiple of 5 bytes")
        self._check(self._L.grg_load_csr5(self._h, num_vars, v_begin, v_begin + len(degree), _ptr(degree),
                                          stream.size // 5, _ptr(stream), 0), "load_csr5")
        self.num_vars = num_vars

    def range_reach(self, v_begin, v_end, label_mask, bounds):
        bounds = np.ascontiguousarray(bounds, dtype=np.uint32)
        out = np.zeros(len(bounds) - 1, np.uint8)
        self._check(self._L.grg_range_reach(self._h, v_begin, v_end, label_mask, len(out), _ptr(bounds), _ptr(out)),
                    "range_reach")
        return out

    def range_counts(self, v_begin, v_end):
        counts = np.zeros(self.num_labels, dtype=np.uint64)
        h = ctypes.c_uint64()
        self._check(self._L.grg_range_counts(self._h, v_begin, v_end, _ptr(counts), ctypes.byref(h)), "range_counts")
        return counts, h.value


def run_closure(num_vars, rules, num_labels, filter_flag, src, dst, lab, device=0, pool_bytes=0, timing=False):
    """Convenience: one context, one closure. Returns (context, stats)."""
    ctx = Context(device)
    ctx.transfer_rules(rules, num_labels)
    ctx.allocate_pool(pool_bytes)
    ctx.set_kernel_timing(timing)
    ctx.load_edges(num_vars, src, dst, lab)
    stats = ctx.closure(filter_flag)
    return ctx, stats


class Partitioned:
    """Out-of-core closure over vertex-range partitions (grg_part_*) on a
    context that holds the grammar (and, optionally, a pool limit)."""

    def __init__(self, ctx: Context, num_vars: int, num_parts: int, restore_from: str | None = None):
        """num_parts equal vertex ranges; or, with restore_from, the partition set
        saved in that checkpoint file (num_vars and num_parts are then ignored)."""
        self.ctx = ctx
        self.num_vars = num_vars
        h = ctypes.c_void_p()
        if restore_from is not None:
            ctx._check(ctx._L.grg_part_restore(ctypes.byref(h), ctx._h, os.fsencode(restore_from)), "part_restore")
        else:
            ctx._check(ctx._L.grg_part_create(ctypes.byref(h), ctx._h, num_vars, num_parts), "part_create")
        self._h = h
        self.paused = False

    def close(self):
        if getattr(self, "_h", None):
            self.ctx._L.grg_part_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def load_edges(self, src, dst, lab):
        src = np.ascontiguousarray(src, dtype=np.uint32)
        dst = np.ascontiguousarray(dst, dtype=np.uint32)
        lab = np.ascontiguousarray(lab, dtype=np.uint8)
        self.ctx._check(self.ctx._L.grg_part_load_edges(self._h, len(src), _ptr(src), _ptr(dst), _ptr(lab)),
                        "part_load_edges")

    def run(self, filter_flag: int) -> dict:
        """This call's statistics; self.paused tells whether the run budget stopped it."""
        s = PartStats()
        st = self.ctx._L.grg_part_run(self._h, filter_flag, ctypes.byref(s))
        if st != PAUSED:
            self.ctx._check(st, "part_run")
        self.paused = st == PAUSED
        return s.as_dict()

    def save(self, path: str):
        self.ctx._check(self.ctx._L.grg_part_save(self._h, os.fsencode(path)), "part_save")

    def set_checkpoint(self, path: str | None, every_runs: int = 1):
        self.ctx._check(self.ctx._L.grg_part_set_checkpoint(self._h, os.fsencode(path) if path else None,
                                                            every_runs), "part_set_checkpoint")

    def set_run_budget(self, max_runs: int):
        self.ctx._check(self.ctx._L.grg_part_set_run_budget(self._h, max_runs), "part_set_run_budget")

    def export_csr5(self, index: int):
        """Partition index's rows as the compressed edge stream (closed sets)."""
        n = ctypes.c_uint64()
        st = self.ctx._L.grg_part_export_csr5(self._h, index, 0, None, None, ctypes.byref(n))
        if st not in (OK, E_RANGE):
            self.ctx._check(st, "part_export_csr5")
        b = self.bounds()
        out = np.zeros(n.value * 5, np.uint8)
        deg = np.zeros(int(b[index + 1] - b[index]), np.uint32)
        self.ctx._check(self.ctx._L.grg_part_export_csr5(self._h, index, n.value, _ptr(out), _ptr(deg),
                                                         ctypes.byref(n)), "part_export_csr5")
        return out, deg

    def label_counts(self):
        counts = np.zeros(self.ctx.num_labels, dtype=np.uint64)
        h = ctypes.c_uint64()
        self.ctx._check(self.ctx._L.grg_part_label_counts(self._h, _ptr(counts), ctypes.byref(h)), "part_label_counts")
        return counts, h.value

    def bounds(self):
        n = ctypes.c_uint32()
        self.ctx._check(self.ctx._L.grg_part_bounds(self._h, 0, None, ctypes.byref(n)), "part_bounds")
        b = np.zeros(n.value + 1, np.uint32)
        self.ctx._check(self.ctx._L.grg_part_bounds(self._h, len(b), _ptr(b), ctypes.byref(n)), "part_bounds")
        return b


class Batch:
    """Many independent closures in one context (grg_batch_*).

    grammars: list of (rules, labels) with rules as tuples of label names (LHS
    first, as in grg_gen). Each grammar gets its own label range in the union
    grammar; a job names its grammar by index and uses that grammar's label ids
    (1-based, first-appearance order)."""

    def __init__(self, ctx: Context, max_vars: int, max_jobs: int, grammars, filter_flag: int = 0):
        self.ctx = ctx
        self.max_jobs = max_jobs
        self.offsets, self.sizes, self.eps = [], [], []
        union = []
        off = 0
        for rules, labels in grammars:
            ids = {n: i + 1 + off for i, n in enumerate(labels)}
            eps = 0
            for r in rules:
                row = [ids[r[0]], ids[r[1]] if len(r) > 1 else 0, ids[r[2]] if len(r) > 2 else 0]
                union.append(row)
                if len(r) == 1:
                    eps |= 1 << (ids[r[0]] - 1)
            self.offsets.append(off)
            self.sizes.append(len(labels))
            self.eps.append(eps)
            off += len(labels)
        self.num_labels = off
        r = np.ascontiguousarray(np.array(union, dtype=np.int32).reshape(-1))
        ctx._check(ctx._L.grg_batch_begin(ctx._h, max_vars, max_jobs, len(r) // 3, _ptr(r), off, filter_flag),
                   "batch_begin")
        self._rec = np.zeros(max_jobs, dtype=np.uint32)

    def admit(self, job: int, base: int, grammar: int, num_vars: int, src, dst, lab):
        """Host arrays with job-local vertex ids and the grammar's label ids."""
        src = np.ascontiguousarray(src, dtype=np.uint32)
        dst = np.ascontiguousarray(dst, dtype=np.uint32)
        lab = np.ascontiguousarray(np.asarray(lab, dtype=np.int64) + self.offsets[grammar], dtype=np.uint8)
        self.ctx._check(self.ctx._L.grg_batch_admit(self.ctx._h, job, base, num_vars, len(src), _ptr(src), _ptr(dst),
                                                    _ptr(lab), 0, self.eps[grammar]), "batch_admit")

    def step(self, max_rounds: int = 1):
        """Returns (records per job slot in the last round, rounds with work)."""
        n = ctypes.c_uint64()
        self.ctx._check(self.ctx._L.grg_batch_step(self.ctx._h, max_rounds, _ptr(self._rec), ctypes.byref(n)),
                        "batch_step")
        return self._rec.copy(), n.value

    def result(self, job: int, grammar: int):
        counts = np.zeros(self.sizes[grammar], dtype=np.uint64)
        h = ctypes.c_uint64()
        self.ctx._check(self.ctx._L.grg_batch_result(self.ctx._h, job, self.offsets[grammar], self.sizes[grammar],
                                                     _ptr(counts), ctypes.byref(h)), "batch_result")
        return counts, h.value

    def release(self, job: int):
        self.ctx._check(self.ctx._L.grg_batch_release(self.ctx._h, job), "batch_release")
