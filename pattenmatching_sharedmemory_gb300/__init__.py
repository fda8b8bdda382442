"""GB300-native PruneJuice pruning pipeline (LCC / CC / PC / TDS / ENUMERATION).

Python mirror of the reference's pattern-matching driver
(src/patternmatching/multiple_label_cpu.{h,cc}: allocate, runPatternMatching,
free) over the C ABI declared in include/pm_gb300.h.  Every compute call goes
to the CUDA kernels in libpm_gb300.so; importing this package fails loudly
when that library has not been built (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libpm_gb300.so"
CLI_PATH = _PKG / "lib" / "patternmatching_gb300"

STEP_NAMES = {0: "START", 1: "END", 2: "LCC0", 3: "LCC", 4: "CC", 5: "PC", 6: "TDS", 7: "ENUMERATION"}

PM_SUCCESS = 0
PM_FAILURE = -1
PM_E_INVALID_ARG = -2
PM_E_IO = -3
PM_E_FORMAT = -4
PM_E_PATTERN_TOO_LARGE = -5
PM_E_ADMISSION_DENIED = -6
PM_E_TIMEOUT = -7
PM_E_DEVICE = -8
PM_E_NO_DEVICE = -9
PM_E_CANCELLED = -10
PM_E_OOM = -11
PM_E_BUSY = -12
PM_E_STATISTICS = -13

# Flags or-ed into a query's variant (pm_gb300.h): the article's
# constraint-order drivers (test_article/CMakeLists.txt:53-73).
PM_ORDER_ENUMERATE = 0x100
PM_ORDER_EFFECTIVENESS = 0x200
PM_ORDER_EARLY_ENUMERATION = 0x400
# The reference's order binaries by name (order_intuitive is the backtrack
# variant without flags).
ORDER_DRIVERS = {"intuitive": 0, "enumerate_intuitive": PM_ORDER_ENUMERATE,
                 "effectiveness": PM_ORDER_EFFECTIVENESS,
                 "enumerate_effectiveness": PM_ORDER_EFFECTIVENESS | PM_ORDER_ENUMERATE,
                 "enumerate_effectiveness_early": PM_ORDER_EFFECTIVENESS | PM_ORDER_ENUMERATE
                 | PM_ORDER_EARLY_ENUMERATION}


class PmError(RuntimeError):
    """A non-zero pm_status_t with the library's last error message."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class AlgoResults(ctypes.Structure):
    _fields_ = [("vertex_eliminated", ctypes.c_uint64), ("edge_eliminated", ctypes.c_uint64),
                ("match_eliminated", ctypes.c_uint64), ("enumeration", ctypes.c_uint64)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("memory_budget", ctypes.c_uint64), ("walk_share", ctypes.c_uint32)]


class RequestResult(ctypes.Structure):
    """pm_request_result: outcome and timings of one served request."""

    _fields_ = [("status", ctypes.c_int32), ("n_records", ctypes.c_int32), ("match_count", ctypes.c_uint64),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("gpu_ms", ctypes.c_double), ("charged_bytes", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_uint64), ("running", ctypes.c_uint64), ("done", ctypes.c_uint64),
                ("bytes_in_use", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64),
                ("memory_budget", ctypes.c_uint64), ("slots", ctypes.c_uint32)]


class TemplateCsr(ctypes.Structure):
    _fields_ = [("offsets", ctypes.POINTER(ctypes.c_uint64)), ("adj", ctypes.POINTER(ctypes.c_uint32)),
                ("labels", ctypes.POINTER(ctypes.c_uint64)), ("vertex_count", ctypes.c_uint32),
                ("edge_count", ctypes.c_uint64)]


class TuneResult(ctypes.Structure):
    """pm_tune_result: the choices pm_autotune left in force."""

    _fields_ = [("hub_degree", ctypes.c_uint32), ("seg_entries", ctypes.c_uint32),
                ("enum_presplit_memo", ctypes.c_uint32), ("enum_presplit_plain", ctypes.c_uint32),
                ("enum_table_entries", ctypes.c_uint32), ("walk_presplit", ctypes.c_uint32),
                ("walk_table_entries", ctypes.c_uint32), ("probes_memo", ctypes.c_uint32),
                ("probes_plain", ctypes.c_uint32), ("runs", ctypes.c_uint32),
                ("enum_tail_swap", ctypes.c_uint32), ("walk_tail_swap", ctypes.c_uint32),
                ("enum_count_memo", ctypes.c_uint32), ("walk_tail_state_memo", ctypes.c_uint32),
                ("enum_pair_tail", ctypes.c_uint32), ("walk_pair_tail", ctypes.c_uint32),
                ("enum_second_split", ctypes.c_uint32)]

    def as_dict(self):
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


PM_SUBMIT_EXPORT_STATE = 1
PM_SUBMIT_PRUNE_ONLY = 2


class StepRecord(ctypes.Structure):
    """One results.totem row (pm_step_record)."""

    _fields_ = [("iteration", ctypes.c_int32), ("step", ctypes.c_int32), ("step_ms", ctypes.c_double),
                ("cumulative_ms", ctypes.c_double), ("results", AlgoResults), ("active_vertex", ctypes.c_uint64),
                ("total_vertex", ctypes.c_uint64), ("active_edge", ctypes.c_uint64),
                ("total_edge", ctypes.c_uint64)]

    def as_tuple(self):
        """The row without its timing columns: (step, vertex eliminated, active vertex, total vertex,
        edge eliminated, active edge, total edge, match eliminated, enumeration)."""
        r = self.results
        return (STEP_NAMES[self.step], r.vertex_eliminated, self.active_vertex, self.total_vertex,
                r.edge_eliminated, self.active_edge, self.total_edge, r.match_eliminated, r.enumeration)


def _load_library() -> ctypes.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build the GB300 extension first "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(str(LIB_PATH))
    P = ctypes.POINTER
    c_u64p, c_u32p, c_u8p = P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint8)
    sig = {
        "pm_last_error": (ctypes.c_char_p, []),
        "pm_version": (ctypes.c_char_p, []),
        "pm_graph_load": (ctypes.c_int32, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                           P(ctypes.c_void_p)]),
        "pm_graph_from_csr": (ctypes.c_int32, [c_u64p, c_u32p, c_u64p, ctypes.c_uint32, ctypes.c_uint64,
                                               ctypes.c_int, P(ctypes.c_void_p)]),
        "pm_graph_store_binary": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p]),
        "pm_graph_info": (ctypes.c_int32, [ctypes.c_void_p, c_u32p, c_u64p, c_u64p]),
        "pm_graph_destroy": (None, [ctypes.c_void_p]),
        "pm_graph_generate_rmat": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                                    ctypes.c_int32, P(ctypes.c_void_p)]),
        "pm_graph_assign_labels": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32,
                                                    ctypes.c_double, ctypes.c_uint64]),
        "pm_graph_host_csr": (ctypes.c_int32, [ctypes.c_void_p, P(c_u64p), P(c_u32p), P(c_u64p)]),
        "pm_graph_make_undirected": (ctypes.c_int32, [ctypes.c_void_p, P(ctypes.c_void_p)]),
        "pm_graph_sort_neighbours": (ctypes.c_int32, [ctypes.c_void_p]),
        "pm_graph_sort_vertices_by_degree": (ctypes.c_int32, [ctypes.c_void_p, P(ctypes.c_void_p), c_u32p]),
        "pm_graph_to_device": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32]),
        "pm_graph_write_text": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]),
        "pm_graph_set_hub_plan": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]),
        "pm_query_create": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, P(ctypes.c_void_p)]),
        "pm_query_create_from_csr": (ctypes.c_int32, [ctypes.c_void_p, c_u64p, c_u32p, c_u64p, ctypes.c_uint32,
                                                      ctypes.c_uint64, P(ctypes.c_void_p)]),
        "pm_query_create_variant": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int32,
                                                     P(ctypes.c_void_p)]),
        "pm_query_create_variant_from_csr": (ctypes.c_int32, [ctypes.c_void_p, c_u64p, c_u32p, c_u64p,
                                                              ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32,
                                                              P(ctypes.c_void_p)]),
        "pm_query_constraint_counts": (ctypes.c_int32, [ctypes.c_void_p, P(ctypes.c_int32), P(ctypes.c_int32),
                                                        P(ctypes.c_int32)]),
        "pm_query_dump_constraints": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t,
                                                       P(ctypes.c_size_t)]),
        "pm_query_step": (ctypes.c_int32, [ctypes.c_void_p, P(StepRecord), P(ctypes.c_int)]),
        "pm_query_run": (ctypes.c_int32, [ctypes.c_void_p, P(StepRecord), ctypes.c_int32, P(ctypes.c_int32)]),
        "pm_query_prune": (ctypes.c_int32, [ctypes.c_void_p, P(StepRecord), ctypes.c_int32, P(ctypes.c_int32)]),
        "pm_set_query_budget_ms": (ctypes.c_int32, [ctypes.c_double]),
        "pm_query_list_matches": (ctypes.c_int32, [ctypes.c_void_p, c_u32p, ctypes.c_uint64, c_u32p, c_u64p]),
        "pm_query_write_matches": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_uint64, c_u64p]),
        "pm_query_export_subgraph": (ctypes.c_int32, [ctypes.c_void_p, c_u64p, c_u32p, ctypes.c_uint64, c_u64p]),
        "pm_debug_fail_device_alloc_after": (ctypes.c_int32, [ctypes.c_int64]),
        "pm_server_cancel": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64]),
        "pm_query_export": (ctypes.c_int32, [ctypes.c_void_p, c_u64p, c_u8p, c_u8p]),
        "pm_query_write_outputs": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p]),
        "pm_query_match_count": (ctypes.c_int32, [ctypes.c_void_p, c_u64p]),
        "pm_query_device_bytes": (ctypes.c_int32, [ctypes.c_void_p, c_u64p]),
        "pm_query_estimate_bytes": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, c_u64p]),
        "pm_query_stats": (ctypes.c_int32, [ctypes.c_void_p, c_u64p, c_u64p]),
        "pm_query_step_walk_stats": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, c_u64p, c_u64p]),
        "pm_device_count": (ctypes.c_int32, []),
        "pm_kernel_launches": (ctypes.c_uint64, []),
        "pm_query_elapsed_ms": (ctypes.c_int32, [ctypes.c_void_p, P(ctypes.c_double)]),
        "pm_set_walk_budget_ms": (ctypes.c_int32, [ctypes.c_double]),
        "pm_set_order_threads": (ctypes.c_int32, [ctypes.c_int32]),
        "pm_query_graph_stat": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint32),
                                                 c_u64p, c_u64p, c_u64p, c_u64p]),
        "pm_query_aborted_step": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64),
                                                   ctypes.POINTER(ctypes.c_uint64)]),
        "pm_set_enum_split": (ctypes.c_int32, [ctypes.c_uint32, ctypes.c_uint32]),
        "pm_set_enum_table_entries": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_set_noalloc_table_entries": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_noalloc_last_rounds": (ctypes.c_uint32, []),
        "pm_set_lcc_graph": (ctypes.c_int32, [ctypes.c_int32]),
        "pm_set_lcc_label_stream": (ctypes.c_int32, [ctypes.c_int32]),
        "pm_set_enum_tail_swap": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_set_walk_tail_swap": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_set_enum_count_memo": (ctypes.c_int32, [ctypes.c_int32]),
        "pm_set_walk_tail_state_memo": (ctypes.c_int32, [ctypes.c_int32]),
        "pm_set_pair_tail": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
        "pm_set_enum_second_split": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_set_walk_table_entries": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_set_walk_presplit": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_set_enum_presplit": (ctypes.c_int32, [ctypes.c_uint32]),
        "pm_set_enum_presplit_by_kind": (ctypes.c_int32, [ctypes.c_uint32, ctypes.c_uint32]),
        "pm_autotune": (ctypes.c_int32, [ctypes.c_void_p, P(TemplateCsr), ctypes.c_uint32, ctypes.c_uint32,
                                         P(TuneResult)]),
        "pm_template_dump_constraints": (ctypes.c_int32, [c_u64p, c_u32p, c_u64p, ctypes.c_uint32, ctypes.c_uint64,
                                                          ctypes.c_char_p, ctypes.c_size_t, P(ctypes.c_size_t)]),
        "pm_query_destroy": (None, [ctypes.c_void_p]),
        "pm_server_create": (ctypes.c_int32, [ctypes.c_void_p, P(ServerConfig), P(ctypes.c_void_p)]),
        "pm_server_submit": (ctypes.c_int32, [ctypes.c_void_p, c_u64p, c_u32p, c_u64p, ctypes.c_uint32,
                                              ctypes.c_uint64, ctypes.c_uint32, c_u64p]),
        "pm_server_poll": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, P(ctypes.c_int), P(RequestResult)]),
        "pm_server_wait": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, P(RequestResult)]),
        "pm_server_records": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, P(StepRecord), ctypes.c_int32,
                                               P(ctypes.c_int32)]),
        "pm_server_export": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, c_u64p, c_u8p, c_u8p]),
        "pm_server_release": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64]),
        "pm_server_stats_get": (ctypes.c_int32, [ctypes.c_void_p, P(ServerStats)]),
        "pm_server_destroy": (None, [ctypes.c_void_p]),
        "pm_batch_run": (ctypes.c_int32, [ctypes.c_void_p, P(TemplateCsr), ctypes.c_uint32, ctypes.c_uint32,
                                          c_u64p, P(ctypes.c_int32)]),
        "pm_fused_batch_run": (ctypes.c_int32, [ctypes.c_void_p, P(TemplateCsr), ctypes.c_uint32, ctypes.c_uint32,
                                                P(ctypes.c_void_p)]),
        "pm_fused_batch_result": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, P(RequestResult)]),
        "pm_fused_batch_records": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, P(StepRecord), ctypes.c_int32,
                                                    P(ctypes.c_int32)]),
        "pm_fused_batch_export": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, c_u64p, c_u8p, c_u8p]),
        "pm_fused_batch_stats": (ctypes.c_int32, [ctypes.c_void_p, c_u64p, c_u64p]),
        "pm_fused_batch_destroy": (None, [ctypes.c_void_p]),
        # Device buffers (d_*) and the stream are passed as raw addresses.
        "pm_enumerate_noalloc": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                                  ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                  c_u64p, c_u32p, c_u64p, ctypes.c_uint32, ctypes.c_uint64,
                                                  ctypes.c_void_p, ctypes.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load_library()

from .templates import Pattern  # noqa: E402  (pure numpy; re-exported here)


def _check(status: int) -> None:
    if status != PM_SUCCESS:
        raise PmError(status, lib.pm_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _enc(s) -> bytes | None:
    if s is None:
        return None
    return os.fsencode(str(s))


class Graph:
    """A labelled CSR graph (TOTEM graph_t) resident on one GPU."""

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    @classmethod
    def load(cls, graph_path, bin_path=None, labels_path=None, device: int = 0) -> "Graph":
        h = ctypes.c_void_p()
        _check(lib.pm_graph_load(_enc(graph_path), _enc(bin_path), _enc(labels_path), device, ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_csr(cls, offsets, adj, labels=None, device: int = 0) -> "Graph":
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        ad = np.ascontiguousarray(adj, dtype=np.uint32)
        lab = None if labels is None else np.ascontiguousarray(labels, dtype=np.uint64)
        h = ctypes.c_void_p()
        _check(lib.pm_graph_from_csr(_ptr(off, ctypes.c_uint64), _ptr(ad, ctypes.c_uint32),
                                     None if lab is None else _ptr(lab, ctypes.c_uint64), len(off) - 1, len(ad),
                                     device, ctypes.byref(h)))
        return cls(h)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1, permute: bool = True) -> "Graph":
        """Seeded undirected RMAT graph (host-only until a query or to_device)."""
        h = ctypes.c_void_p()
        _check(lib.pm_graph_generate_rmat(scale, edge_factor, a, b, c, seed, int(permute), ctypes.byref(h)))
        return cls(h)

    def assign_labels(self, kind: str, n_labels: int, s: float = 1.0, seed: int = 1) -> "Graph":
        k = {"uniform": 0, "zipf": 1, "degree": 2}[kind]
        _check(lib.pm_graph_assign_labels(self._h, k, n_labels, s, seed))
        return self

    def to_device(self, device: int = 0) -> "Graph":
        _check(lib.pm_graph_to_device(self._h, device))
        return self

    def set_hub_plan(self, hub_degree: int, seg_entries: int) -> "Graph":
        """LCC degree classes: lists longer than hub_degree are split into
        seg_entries-entry segments (speed only; results do not change)."""
        _check(lib.pm_graph_set_hub_plan(self._h, hub_degree, seg_entries))
        return self

    @property
    def vertex_count(self) -> int:
        v = ctypes.c_uint32()
        _check(lib.pm_graph_info(self._h, ctypes.byref(v), None, None))
        return v.value

    @property
    def edge_count(self) -> int:
        e = ctypes.c_uint64()
        _check(lib.pm_graph_info(self._h, None, ctypes.byref(e), None))
        return e.value

    @property
    def device_bytes(self) -> int:
        b = ctypes.c_uint64()
        _check(lib.pm_graph_info(self._h, None, None, ctypes.byref(b)))
        return b.value

    def host_csr(self):
        """Zero-copy numpy views of the library-owned host CSR: (offsets, adj, labels)."""
        o, a, l = ctypes.POINTER(ctypes.c_uint64)(), ctypes.POINTER(ctypes.c_uint32)(), ctypes.POINTER(ctypes.c_uint64)()
        _check(lib.pm_graph_host_csr(self._h, ctypes.byref(o), ctypes.byref(a), ctypes.byref(l)))
        V, E = self.vertex_count, self.edge_count
        off = np.ctypeslib.as_array(o, shape=(V + 1,)) if V + 1 else np.zeros(0, np.uint64)
        adj = np.ctypeslib.as_array(a, shape=(E,)) if E else np.zeros(0, np.uint32)
        lab = np.ctypeslib.as_array(l, shape=(V,)) if V and l else np.zeros(V, np.uint64)
        return off, adj, lab

    def undirected(self) -> "Graph":
        """The generator's UNDIRECTED command: a new host graph with every
        entry in both directions (duplicates kept)."""
        h = ctypes.c_void_p()
        _check(lib.pm_graph_make_undirected(self._h, ctypes.byref(h)))
        return Graph(h)

    def sort_neighbours(self) -> "Graph":
        """The generator's SORT_NEIGHBOURS command, in place."""
        _check(lib.pm_graph_sort_neighbours(self._h))
        return self

    def sorted_by_degree(self):
        """The generator's SORT_VERTICES command: (new host graph, old_to_new)."""
        h = ctypes.c_void_p()
        m = np.zeros(max(self.vertex_count, 1), np.uint32)
        _check(lib.pm_graph_sort_vertices_by_degree(self._h, ctypes.byref(h), _ptr(m, ctypes.c_uint32)))
        return Graph(h), m[:self.vertex_count]

    def write_text(self, graph_path, labels_path=None) -> None:
        _check(lib.pm_graph_write_text(self._h, _enc(graph_path), _enc(labels_path)))

    def store_binary(self, path) -> None:
        _check(lib.pm_graph_store_binary(self._h, _enc(path)))

    def close(self) -> None:
        if self._h:
            lib.pm_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Query:
    """One template over a resident graph: constraint generation, GPU pruning
    steps and the reference's step schedule (MultipleLabelCpu)."""

    VARIANTS = {None: 0, "reference": 0, "strict": 1, "backtrack": 2}

    def __init__(self, graph: Graph, pattern_dir=None, pattern: Pattern | None = None,
                 load_pattern_labels: bool = True, variant: str | None = None, order: int | str = 0):
        """variant: None / "reference" (the reference's walks), or the article
        drivers' "strict" / "backtrack" walks (pm_query_create_variant*).
        order: PM_ORDER_* flags, or an order driver's name (ORDER_DRIVERS), for
        the article's constraint-order drivers (strict / backtrack walks)."""
        self.graph = graph
        self._h = ctypes.c_void_p()
        self._k = None if pattern is None else pattern.n
        v = self.VARIANTS[variant] | (ORDER_DRIVERS[order] if isinstance(order, str) else int(order))
        if pattern_dir is not None:
            d = str(pattern_dir)
            _check(lib.pm_query_create_variant(graph._h, _enc(d), int(load_pattern_labels), v, ctypes.byref(self._h)))
        else:
            p = pattern
            off = np.ascontiguousarray(p.offsets, np.uint64)
            adj = np.ascontiguousarray(p.adj, np.uint32)
            lab = np.ascontiguousarray(p.labels, np.uint64)
            _check(lib.pm_query_create_variant_from_csr(graph._h, _ptr(off, ctypes.c_uint64),
                                                        _ptr(adj, ctypes.c_uint32), _ptr(lab, ctypes.c_uint64), p.n,
                                                        len(adj), v, ctypes.byref(self._h)))

    def constraint_counts(self):
        a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _check(lib.pm_query_constraint_counts(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def dump_constraints(self) -> str:
        need = ctypes.c_size_t()
        _check(lib.pm_query_dump_constraints(self._h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        _check(lib.pm_query_dump_constraints(self._h, buf, need.value, None))
        return buf.value.decode()

    def step(self):
        rec = StepRecord()
        fin = ctypes.c_int()
        _check(lib.pm_query_step(self._h, ctypes.byref(rec), ctypes.byref(fin)))
        return rec, bool(fin.value)

    def run(self) -> list[StepRecord]:
        cap = 1100
        recs = (StepRecord * cap)()
        n = ctypes.c_int32()
        _check(lib.pm_query_run(self._h, recs, cap, ctypes.byref(n)))
        return [recs[i] for i in range(min(n.value, cap))]

    def prune(self) -> list[StepRecord]:
        """pm_query_prune: the pipeline up to (not including) ENUMERATION."""
        cap = 1100
        recs = (StepRecord * cap)()
        n = ctypes.c_int32()
        _check(lib.pm_query_prune(self._h, recs, cap, ctypes.byref(n)))
        return [recs[i] for i in range(min(n.value, cap))]

    def export(self):
        V, E = self.graph.vertex_count, self.graph.edge_count
        cand = np.zeros(V, np.uint64)
        eact = np.zeros(E, np.uint8)
        vact = np.zeros(V, np.uint8)
        _check(lib.pm_query_export(self._h, _ptr(cand, ctypes.c_uint64), _ptr(eact, ctypes.c_uint8),
                                   _ptr(vact, ctypes.c_uint8)))
        return cand, eact, vact

    def list_matches(self, cap: int = 1 << 20):
        """pm_query_list_matches: (matches as an (n, k) uint32 array, at most
        cap rows; total count)."""
        per, n = ctypes.c_uint32(), ctypes.c_uint64()
        k = self._k
        if k is None:  # template from files: ask for the match width first
            _check(lib.pm_query_list_matches(self._h, None, 0, ctypes.byref(per), ctypes.byref(n)))
            k = per.value
        buf = np.zeros(max(cap, 1) * max(k, 1), np.uint32)
        _check(lib.pm_query_list_matches(self._h, _ptr(buf, ctypes.c_uint32), cap, ctypes.byref(per),
                                         ctypes.byref(n)))
        rows = min(n.value, cap)
        return buf[:rows * per.value].reshape(rows, per.value), n.value

    def write_matches(self, path, max_matches: int = 1 << 20) -> int:
        n = ctypes.c_uint64()
        _check(lib.pm_query_write_matches(self._h, _enc(path), max_matches, ctypes.byref(n)))
        return n.value

    def export_subgraph(self):
        """pm_query_export_subgraph: (offsets[V + 1], adj) of the pruned subgraph."""
        V = self.graph.vertex_count
        off = np.zeros(V + 1, np.uint64)
        n = ctypes.c_uint64()
        _check(lib.pm_query_export_subgraph(self._h, _ptr(off, ctypes.c_uint64), None, 0, ctypes.byref(n)))
        adj = np.zeros(max(n.value, 1), np.uint32)
        _check(lib.pm_query_export_subgraph(self._h, None, _ptr(adj, ctypes.c_uint32), n.value, ctypes.byref(n)))
        return off, adj[:n.value]

    def write_outputs(self, out_dir) -> None:
        _check(lib.pm_query_write_outputs(self._h, _enc(out_dir)))

    @property
    def match_count(self) -> int:
        c = ctypes.c_uint64()
        _check(lib.pm_query_match_count(self._h, ctypes.byref(c)))
        return c.value

    @property
    def device_bytes(self) -> int:
        b = ctypes.c_uint64()
        _check(lib.pm_query_device_bytes(self._h, ctypes.byref(b)))
        return b.value

    def stats(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib.pm_query_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return {"exact_resolutions": a.value, "overflow_retries": b.value}

    @property
    def elapsed_ms(self) -> float:
        """Device time from the start of the first step to the end of the latest."""
        ms = ctypes.c_double()
        _check(lib.pm_query_elapsed_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def graph_stat(self, threads: int = 1):
        """pm_query_graph_stat: (labels, vertex_total[n], edge_total[n, n],
        at_least[n, n, 64]) of the query's current state, taken on the GPU."""
        n = ctypes.c_uint32()
        labs = np.zeros(64, np.uint64)
        vt = np.zeros(64, np.uint64)
        et = np.zeros(64 * 64, np.uint64)
        al = np.zeros(64 * 64 * 64, np.uint64)
        _check(lib.pm_query_graph_stat(self._h, int(threads), ctypes.byref(n), _ptr(labs, ctypes.c_uint64),
                                       _ptr(vt, ctypes.c_uint64), _ptr(et, ctypes.c_uint64), _ptr(al, ctypes.c_uint64)))
        k = n.value
        return labs[:k], vt[:k], et[:k * k].reshape(k, k), al[:k * k * 64].reshape(k, k, 64)

    def aborted_step(self):
        """(step kind, device ms, CSR entries tested, hops) of the step that
        ended the run with PM_E_TIMEOUT (pm_query_aborted_step), or None."""
        k, ms, a, b = ctypes.c_int32(), ctypes.c_double(), ctypes.c_uint64(), ctypes.c_uint64()
        if lib.pm_query_aborted_step(self._h, ctypes.byref(k), ctypes.byref(ms), ctypes.byref(a),
                                     ctypes.byref(b)) != PM_SUCCESS:
            return None
        return k.value, ms.value, a.value, b.value

    def step_walk_stats(self, row: int):
        """(CSR entries tested, hops taken) by the walkers of result row `row`."""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib.pm_query_step_walk_stats(self._h, row, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def close(self) -> None:
        if self._h:
            lib.pm_query_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous batching of template queries over one resident graph
    (pm_server_*): `slots` queries run on the GPU at once, admitted in FIFO
    order as slots and the device-memory budget allow."""

    def __init__(self, graph: Graph, slots: int = 4, memory_budget: int = 0, walk_share: int = 0):
        """walk_share: pm_server_config.walk_share (0: 1/slots of the GPU
        per slot's walker launches, 1: the whole GPU)."""
        self.graph = graph
        self._h = ctypes.c_void_p()
        cfg = ServerConfig(slots, memory_budget, walk_share)
        _check(lib.pm_server_create(graph._h, ctypes.byref(cfg), ctypes.byref(self._h)))

    def submit(self, pattern: Pattern, export_state: bool = False, prune_only: bool = False) -> int:
        off = np.ascontiguousarray(pattern.offsets, np.uint64)
        adj = np.ascontiguousarray(pattern.adj, np.uint32)
        lab = np.ascontiguousarray(pattern.labels, np.uint64)
        t = ctypes.c_uint64()
        flags = (PM_SUBMIT_EXPORT_STATE if export_state else 0) | (PM_SUBMIT_PRUNE_ONLY if prune_only else 0)
        _check(lib.pm_server_submit(self._h, _ptr(off, ctypes.c_uint64), _ptr(adj, ctypes.c_uint32),
                                    _ptr(lab, ctypes.c_uint64), pattern.n, len(adj), flags, ctypes.byref(t)))
        return t.value

    def poll(self, ticket: int) -> RequestResult | None:
        done = ctypes.c_int()
        r = RequestResult()
        _check(lib.pm_server_poll(self._h, ticket, ctypes.byref(done), ctypes.byref(r)))
        return r if done.value else None

    def wait(self, ticket: int, timeout_ms: float = -1.0) -> RequestResult:
        r = RequestResult()
        _check(lib.pm_server_wait(self._h, ticket, timeout_ms, ctypes.byref(r)))
        return r

    def records(self, ticket: int) -> list[StepRecord]:
        n = ctypes.c_int32()
        _check(lib.pm_server_records(self._h, ticket, None, 0, ctypes.byref(n)))
        recs = (StepRecord * max(n.value, 1))()
        _check(lib.pm_server_records(self._h, ticket, recs, n.value, ctypes.byref(n)))
        return [recs[i] for i in range(n.value)]

    def export(self, ticket: int):
        V, E = self.graph.vertex_count, self.graph.edge_count
        cand = np.zeros(V, np.uint64)
        eact = np.zeros(E, np.uint8)
        vact = np.zeros(V, np.uint8)
        _check(lib.pm_server_export(self._h, ticket, _ptr(cand, ctypes.c_uint64), _ptr(eact, ctypes.c_uint8),
                                    _ptr(vact, ctypes.c_uint8)))
        return cand, eact, vact

    def cancel(self, ticket: int) -> None:
        """pm_server_cancel: a queued request ends at once, a running one
        before its next step (status PM_E_CANCELLED)."""
        _check(lib.pm_server_cancel(self._h, ticket))

    def release(self, ticket: int) -> None:
        _check(lib.pm_server_release(self._h, ticket))

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(lib.pm_server_stats_get(self._h, ctypes.byref(st)))
        return st

    def close(self) -> None:
        if self._h:
            lib.pm_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _template_array(patterns):
    keep = []
    arr = (TemplateCsr * max(len(patterns), 1))()
    for i, p in enumerate(patterns):
        off = np.ascontiguousarray(p.offsets, np.uint64)
        adj = np.ascontiguousarray(p.adj, np.uint32)
        lab = np.ascontiguousarray(p.labels, np.uint64)
        keep += [off, adj, lab]
        arr[i] = TemplateCsr(_ptr(off, ctypes.c_uint64), _ptr(adj, ctypes.c_uint32), _ptr(lab, ctypes.c_uint64),
                             p.n, len(adj))
    return arr, keep


def autotune(graph: Graph, patterns, max_per_group: int = 4) -> dict:
    """pm_autotune: times candidate degree classes and enumeration settings
    on the probe templates, keeps the fastest in force, returns them."""
    arr, keep = _template_array(patterns)
    r = TuneResult()
    _check(lib.pm_autotune(graph._h, arr, len(patterns), max_per_group, ctypes.byref(r)))
    del keep
    return r.as_dict()


def batch_run(graph: Graph, patterns, slots: int = 4):
    """pm_batch_run: every template's match count and status, `slots` at a time."""
    keep = []
    arr = (TemplateCsr * max(len(patterns), 1))()
    for i, p in enumerate(patterns):
        off = np.ascontiguousarray(p.offsets, np.uint64)
        adj = np.ascontiguousarray(p.adj, np.uint32)
        lab = np.ascontiguousarray(p.labels, np.uint64)
        keep += [off, adj, lab]
        arr[i] = TemplateCsr(_ptr(off, ctypes.c_uint64), _ptr(adj, ctypes.c_uint32), _ptr(lab, ctypes.c_uint64),
                             p.n, len(adj))
    counts = np.zeros(len(patterns), np.uint64)
    statuses = np.zeros(len(patterns), np.int32)
    _check(lib.pm_batch_run(graph._h, arr, len(patterns), slots, _ptr(counts, ctypes.c_uint64),
                            _ptr(statuses, ctypes.c_int32)))
    return counts, statuses


class FusedBatch:
    """pm_fused_batch_run: the templates run as one batch in lockstep rounds,
    their LCC work in shared multi-query launches; per-query results equal
    each template run on its own."""

    def __init__(self, graph: Graph, patterns, prune_only: bool = False):
        self.graph = graph
        self.n = len(patterns)
        arr, keep = _template_array(patterns)
        self._h = ctypes.c_void_p()
        flags = PM_SUBMIT_PRUNE_ONLY if prune_only else 0
        _check(lib.pm_fused_batch_run(graph._h, arr, len(patterns), flags, ctypes.byref(self._h)))
        del keep

    def result(self, i: int) -> RequestResult:
        r = RequestResult()
        _check(lib.pm_fused_batch_result(self._h, i, ctypes.byref(r)))
        return r

    def records(self, i: int) -> list[StepRecord]:
        n = ctypes.c_int32()
        _check(lib.pm_fused_batch_records(self._h, i, None, 0, ctypes.byref(n)))
        recs = (StepRecord * max(n.value, 1))()
        _check(lib.pm_fused_batch_records(self._h, i, recs, n.value, ctypes.byref(n)))
        return [recs[j] for j in range(n.value)]

    def export(self, i: int):
        V, E = self.graph.vertex_count, self.graph.edge_count
        cand = np.zeros(V, np.uint64)
        eact = np.zeros(E, np.uint8)
        vact = np.zeros(V, np.uint8)
        _check(lib.pm_fused_batch_export(self._h, i, _ptr(cand, ctypes.c_uint64), _ptr(eact, ctypes.c_uint8),
                                         _ptr(vact, ctypes.c_uint8)))
        return cand, eact, vact

    def stats(self) -> dict:
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib.pm_fused_batch_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return {"rounds": a.value, "shared_lcc_phases": b.value}

    def close(self) -> None:
        if self._h:
            lib.pm_fused_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_order_threads(threads: int) -> None:
    """The order drivers' thread count for queries created from now on
    (pm_set_order_threads)."""
    _check(lib.pm_set_order_threads(int(threads)))


def version() -> str:
    return lib.pm_version().decode()


def device_count() -> int:
    return int(lib.pm_device_count())
