"""ORACLE — test infrastructure only.

ctypes wrapper of oracle/pm_oracle.cc, the CPU restatement of the reference's
pattern-matching pipeline.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module; the product never does.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libpm_oracle.so"
REF_BIN = HERE / "_ref" / "patternmatching"


def build() -> Path:
    """Compiles the restatement (g++, a few seconds)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "lib"], check=True)
    return LIB_PATH


class _Record(ctypes.Structure):
    _fields_ = [("iteration", ctypes.c_int32), ("step", ctypes.c_int32), ("step_ms", ctypes.c_double),
                ("cumulative_ms", ctypes.c_double), ("vertex_eliminated", ctypes.c_uint64),
                ("edge_eliminated", ctypes.c_uint64), ("match_eliminated", ctypes.c_uint64),
                ("enumeration", ctypes.c_uint64), ("active_vertex", ctypes.c_uint64),
                ("total_vertex", ctypes.c_uint64), ("active_edge", ctypes.c_uint64), ("total_edge", ctypes.c_uint64)]


class _Options(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("nlcc_threads", ctypes.c_int32),
                ("stop_before_enumeration", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("sample_stride", ctypes.c_int64), ("enum_sample_stride", ctypes.c_int64),
                ("deadline_ms", ctypes.c_double), ("max_steps", ctypes.c_int64), ("order", ctypes.c_int32),
                ("order_threads", ctypes.c_int32)]


STEP_NAMES = {0: "START", 1: "END", 2: "LCC0", 3: "LCC", 4: "CC", 5: "PC", 6: "TDS", 7: "ENUMERATION"}
TIMEOUT = -7
STATISTICS = -13

_lib = None


def _load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        lib = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.POINTER
        lib.pmo_run.restype = ctypes.c_int
        lib.pmo_run.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64), ctypes.c_uint32,
                                ctypes.c_uint64, P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64),
                                ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int64, P(_Record),
                                ctypes.c_int32, P(ctypes.c_int32), P(ctypes.c_uint64), P(ctypes.c_uint8),
                                P(ctypes.c_uint8)]
        lib.pmo_run_ex.restype = ctypes.c_int
        lib.pmo_run_ex.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64), ctypes.c_uint32,
                                   ctypes.c_uint64, P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64),
                                   ctypes.c_uint32, P(_Options), P(_Record), ctypes.c_int32, P(ctypes.c_int32),
                                   P(ctypes.c_uint64), P(ctypes.c_uint8), P(ctypes.c_uint8)]
        lib.pmo_generate_graph.restype = ctypes.c_int
        lib.pmo_generate_graph.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64,
                                           P(ctypes.c_void_p)]
        lib.pmo_graph_csr.restype = ctypes.c_int
        lib.pmo_graph_csr.argtypes = [ctypes.c_void_p, P(ctypes.c_uint32), P(ctypes.c_uint64), P(P(ctypes.c_uint64)),
                                      P(P(ctypes.c_uint32)), P(P(ctypes.c_uint64))]
        lib.pmo_graph_free.restype = None
        lib.pmo_graph_free.argtypes = [ctypes.c_void_p]
        lib.pmo_list_matches.restype = ctypes.c_int
        lib.pmo_list_matches.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64), ctypes.c_uint32,
                                         ctypes.c_uint64, P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64),
                                         ctypes.c_uint32, P(ctypes.c_uint32), ctypes.c_uint64, P(ctypes.c_uint64)]
        lib.pmo_enumerate_state.restype = ctypes.c_int
        lib.pmo_enumerate_state.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64),
                                            ctypes.c_uint32, ctypes.c_uint64, P(ctypes.c_uint64), P(ctypes.c_uint32),
                                            P(ctypes.c_uint64), ctypes.c_uint32, P(ctypes.c_uint64),
                                            P(ctypes.c_uint8), ctypes.c_int64, ctypes.c_int, P(ctypes.c_uint64)]
        lib.pmo_graph_stat.restype = ctypes.c_int
        lib.pmo_graph_stat.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64), ctypes.c_uint32,
                                       ctypes.c_uint64, P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64),
                                       ctypes.c_uint32, P(ctypes.c_uint64), P(ctypes.c_uint8), ctypes.c_int32,
                                       P(ctypes.c_uint32), P(ctypes.c_uint64), P(ctypes.c_uint64),
                                       P(ctypes.c_uint64), P(ctypes.c_uint64)]
        lib.pmo_enumeration_start_role.restype = ctypes.c_int
        lib.pmo_enumeration_start_role.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64),
                                                   ctypes.c_uint32]
        lib.pmo_dump_constraints.restype = ctypes.c_int
        lib.pmo_dump_constraints.argtypes = [P(ctypes.c_uint64), P(ctypes.c_uint32), P(ctypes.c_uint64),
                                             ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t,
                                             P(ctypes.c_size_t)]
        _lib = lib
    return _lib


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


class OracleResult:
    def __init__(self, rows, cand, eact, vact):
        self.rows = rows          # list of tuples without timing (see row_tuple)
        self.timings = []         # per-row step ms
        self.cand = cand
        self.eact = eact
        self.vact = vact

    @property
    def match_count(self) -> int:
        for r in self.rows:
            if r[0] == "ENUMERATION":
                return r[8]
        return 0


def run(offsets, adj, labels, p_offsets, p_adj, p_labels, threads: int = 1, stop_before_enumeration: bool = False,
        sample_stride: int = 1) -> OracleResult:
    """Runs the restated pipeline; threads=1 is the canonical sequential order.
    sample_stride > 1 is a timing sample (CC/PC/TDS/ENUMERATION visit only
    sources with id % stride == 0); its results are not the pipeline's."""
    lib = _load()
    off = np.ascontiguousarray(offsets, np.uint64)
    ad = np.ascontiguousarray(adj, np.uint32)
    lab = np.ascontiguousarray(labels, np.uint64)
    po = np.ascontiguousarray(p_offsets, np.uint64)
    pa = np.ascontiguousarray(p_adj, np.uint32)
    pl = np.ascontiguousarray(p_labels, np.uint64)
    V, E, k = len(off) - 1, len(ad), len(po) - 1
    cap = 1100
    recs = (_Record * cap)()
    n = ctypes.c_int32()
    cand = np.zeros(V, np.uint64)
    eact = np.zeros(E, np.uint8)
    vact = np.zeros(V, np.uint8)
    st = lib.pmo_run(_p(off, ctypes.c_uint64), _p(ad, ctypes.c_uint32), _p(lab, ctypes.c_uint64), V, E,
                     _p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32), _p(pl, ctypes.c_uint64), k, threads,
                     int(stop_before_enumeration), sample_stride, recs, cap, ctypes.byref(n),
                     _p(cand, ctypes.c_uint64), _p(eact, ctypes.c_uint8), _p(vact, ctypes.c_uint8))
    if st != 0:
        raise RuntimeError(f"oracle failed with status {st}")
    rows = [row_tuple(recs[i]) for i in range(n.value)]
    res = OracleResult(rows, cand, eact, vact)
    res.timings = [recs[i].step_ms for i in range(n.value)]
    return res


class OracleTimeout(RuntimeError):
    """The run passed its wall-clock deadline (run_ex deadline_ms)."""


def run_ex(offsets, adj, labels, p_offsets, p_adj, p_labels, threads: int = 1, nlcc_threads: int = 1,
           stop_before_enumeration: bool = False, sample_stride: int = 1, enum_sample_stride: int = 1,
           deadline_ms: float = 0.0, want_state: bool = True, variant: int = 0,
           max_steps: int = 0, order: int = 0, order_threads: int = 1) -> OracleResult:
    """run() with separate thread counts for the LCC sweeps (deterministic in
    any order) and for the CC/PC/TDS/ENUMERATION source loops (1 = the
    canonical order of the alreadyMatched shortcut), an ENUMERATION-only
    source sample (enum_sample_stride > 1: the count over sources
    v % stride == 0, pruning unchanged) and a wall-clock deadline (raises
    OracleTimeout past it).  variant 1 / 2: the reference's article drivers
    with strict / backtrack constraint walks (pruning only, END row).
    order: PM_ORDER_* bits (the article's constraint-order drivers, with
    variant 1 or 2), order_threads their OpenMP thread count; a run the
    reference would abort on an absent graph statistic raises StatMissing."""
    lib = _load()
    off = np.ascontiguousarray(offsets, np.uint64)
    ad = np.ascontiguousarray(adj, np.uint32)
    lab = np.ascontiguousarray(labels, np.uint64)
    po = np.ascontiguousarray(p_offsets, np.uint64)
    pa = np.ascontiguousarray(p_adj, np.uint32)
    pl = np.ascontiguousarray(p_labels, np.uint64)
    V, E, k = len(off) - 1, len(ad), len(po) - 1
    cap = 1100
    recs = (_Record * cap)()
    n = ctypes.c_int32()
    cand = np.zeros(V, np.uint64) if want_state else None
    eact = np.zeros(E, np.uint8) if want_state else None
    vact = np.zeros(V, np.uint8) if want_state else None
    opt = _Options(threads, nlcc_threads, int(stop_before_enumeration), variant, sample_stride, enum_sample_stride,
                   deadline_ms, max_steps, order, order_threads)
    st = lib.pmo_run_ex(_p(off, ctypes.c_uint64), _p(ad, ctypes.c_uint32), _p(lab, ctypes.c_uint64), V, E,
                        _p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32), _p(pl, ctypes.c_uint64), k,
                        ctypes.byref(opt), recs, cap, ctypes.byref(n),
                        _p(cand, ctypes.c_uint64) if want_state else None,
                        _p(eact, ctypes.c_uint8) if want_state else None,
                        _p(vact, ctypes.c_uint8) if want_state else None)
    if st == TIMEOUT:
        raise OracleTimeout(f"oracle run passed its {deadline_ms:.0f} ms deadline")
    if st == STATISTICS:
        raise StatMissing("a graph statistic the dynamic order reads is absent")
    if st != 0:
        raise RuntimeError(f"oracle failed with status {st}")
    rows = [row_tuple(recs[i]) for i in range(n.value)]
    res = OracleResult(rows, cand, eact, vact)
    res.timings = [recs[i].step_ms for i in range(n.value)]
    return res


def graph_stat(offsets, adj, labels, p_offsets, p_adj, p_labels, cand, eact, threads: int = 1):
    """GraphStatCpu::compute over a given state (role mask per vertex, active
    flag per CSR entry) with `threads` static-schedule blocks: (labels,
    vertex_total[n], edge_total[n, n], at_least[n, n, 64]) in the layout of
    the product's pm_query_graph_stat."""
    lib = _load()
    off = np.ascontiguousarray(offsets, np.uint64)
    ad = np.ascontiguousarray(adj, np.uint32)
    lab = np.ascontiguousarray(labels, np.uint64)
    po = np.ascontiguousarray(p_offsets, np.uint64)
    pa = np.ascontiguousarray(p_adj, np.uint32)
    pl = np.ascontiguousarray(p_labels, np.uint64)
    c = np.ascontiguousarray(cand, np.uint64)
    e = np.ascontiguousarray(eact, np.uint8)
    n = ctypes.c_uint32()
    labs = np.zeros(64, np.uint64)
    vt = np.zeros(64, np.uint64)
    et = np.zeros(64 * 64, np.uint64)
    al = np.zeros(64 * 64 * 64, np.uint64)
    st = lib.pmo_graph_stat(_p(off, ctypes.c_uint64), _p(ad, ctypes.c_uint32), _p(lab, ctypes.c_uint64), len(off) - 1,
                            len(ad), _p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32), _p(pl, ctypes.c_uint64),
                            len(po) - 1, _p(c, ctypes.c_uint64), _p(e, ctypes.c_uint8), threads, ctypes.byref(n),
                            _p(labs, ctypes.c_uint64), _p(vt, ctypes.c_uint64), _p(et, ctypes.c_uint64),
                            _p(al, ctypes.c_uint64))
    if st == STATISTICS:
        raise StatMissing("a graph statistic lookup of the reference would throw")
    if st != 0:
        raise RuntimeError(f"oracle failed with status {st}")
    k = n.value
    return labs[:k], vt[:k], et[:k * k].reshape(k, k), al[:k * k * 64].reshape(k, k, 64)


class StatMissing(RuntimeError):
    """The dynamic order read a graph statistic the pruned graph lacks (the
    reference's order driver throws std::out_of_range there and aborts)."""


class HostGraph:
    """A seeded RMAT graph generated inside the oracle library (the
    product's generator source compiled in), so a caller gets the bench
    graph without loading the product library.  offsets / adj / labels are
    numpy views valid while this object lives."""

    def __init__(self, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
                 seed: int = 1, permute: bool = True, label_kind: str = "uniform", n_labels: int = 5,
                 zipf_s: float = 1.0, label_seed: int = 1):
        lib = _load()
        kind = {"uniform": 0, "zipf": 1, "degree": 2}[label_kind]
        h = ctypes.c_void_p()
        st = lib.pmo_generate_graph(scale, edge_factor, a, b, c, seed, int(permute), kind, n_labels, zipf_s,
                                    label_seed, ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"oracle graph generation failed with status {st}")
        self._h = h
        V, E = ctypes.c_uint32(), ctypes.c_uint64()
        o, a_, l = ctypes.POINTER(ctypes.c_uint64)(), ctypes.POINTER(ctypes.c_uint32)(), \
            ctypes.POINTER(ctypes.c_uint64)()
        lib.pmo_graph_csr(h, ctypes.byref(V), ctypes.byref(E), ctypes.byref(o), ctypes.byref(a_), ctypes.byref(l))
        self.vertex_count, self.edge_count = V.value, E.value
        self.offsets = np.ctypeslib.as_array(o, shape=(V.value + 1,))
        self.adj = np.ctypeslib.as_array(a_, shape=(E.value,)) if E.value else np.zeros(0, np.uint32)
        self.labels = np.ctypeslib.as_array(l, shape=(V.value,)) if V.value else np.zeros(0, np.uint64)

    def close(self):
        if self._h:
            _load().pmo_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def row_tuple(r) -> tuple:
    return (STEP_NAMES[r.step], r.vertex_eliminated, r.active_vertex, r.total_vertex, r.edge_eliminated,
            r.active_edge, r.total_edge, r.match_eliminated, r.enumeration)


def list_matches(offsets, adj, labels, p_offsets, p_adj, p_labels, cap: int = 1 << 20):
    """(matches as an (n, k) uint32 array of at most cap rows, total count):
    the embeddings ENUMERATION counts, each as the vertices bound by the
    enumeration walk's vertex moves in walk order."""
    lib = _load()
    off = np.ascontiguousarray(offsets, np.uint64)
    ad = np.ascontiguousarray(adj, np.uint32)
    lab = np.ascontiguousarray(labels, np.uint64)
    po = np.ascontiguousarray(p_offsets, np.uint64)
    pa = np.ascontiguousarray(p_adj, np.uint32)
    pl = np.ascontiguousarray(p_labels, np.uint64)
    k = len(po) - 1
    out = np.zeros(cap * k, np.uint32)
    n = ctypes.c_uint64()
    st = lib.pmo_list_matches(_p(off, ctypes.c_uint64), _p(ad, ctypes.c_uint32), _p(lab, ctypes.c_uint64),
                              len(off) - 1, len(ad), _p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32),
                              _p(pl, ctypes.c_uint64), k, _p(out, ctypes.c_uint32), cap, ctypes.byref(n))
    if st != 0:
        raise RuntimeError(f"oracle listing failed with status {st}")
    rows = min(n.value, cap)
    return out[:rows * k].reshape(rows, k), n.value


def enumerate_state(offsets, adj, labels, p_offsets, p_adj, p_labels, cand, eact, stride: int = 1,
                    threads: int = 1) -> int:
    """ENUMERATION over a given pruned state (role masks, per-CSR-entry
    flags), counting only sources v % stride == 0."""
    lib = _load()
    off = np.ascontiguousarray(offsets, np.uint64)
    ad = np.ascontiguousarray(adj, np.uint32)
    lab = np.ascontiguousarray(labels, np.uint64)
    po = np.ascontiguousarray(p_offsets, np.uint64)
    pa = np.ascontiguousarray(p_adj, np.uint32)
    pl = np.ascontiguousarray(p_labels, np.uint64)
    c = np.ascontiguousarray(cand, np.uint64)
    e = np.ascontiguousarray(eact, np.uint8)
    n = ctypes.c_uint64()
    st = lib.pmo_enumerate_state(_p(off, ctypes.c_uint64), _p(ad, ctypes.c_uint32), _p(lab, ctypes.c_uint64),
                                 len(off) - 1, len(ad), _p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32),
                                 _p(pl, ctypes.c_uint64), len(po) - 1, _p(c, ctypes.c_uint64), _p(e, ctypes.c_uint8),
                                 stride, threads, ctypes.byref(n))
    if st != 0:
        raise RuntimeError(f"oracle enumeration failed with status {st}")
    return n.value


def enumeration_start_role(p_offsets, p_adj, p_labels) -> int:
    """The template vertex whose holders are ENUMERATION's sources."""
    lib = _load()
    po = np.ascontiguousarray(p_offsets, np.uint64)
    pa = np.ascontiguousarray(p_adj, np.uint32)
    pl = np.ascontiguousarray(p_labels, np.uint64)
    r = lib.pmo_enumeration_start_role(_p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32), _p(pl, ctypes.c_uint64),
                                       len(po) - 1)
    if r < 0:
        raise RuntimeError(f"no enumeration walk (status {r})")
    return r


def dump_constraints(p_offsets, p_adj, p_labels) -> str:
    lib = _load()
    po = np.ascontiguousarray(p_offsets, np.uint64)
    pa = np.ascontiguousarray(p_adj, np.uint32)
    pl = np.ascontiguousarray(p_labels, np.uint64)
    k = len(po) - 1
    need = ctypes.c_size_t()
    st = lib.pmo_dump_constraints(_p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32), _p(pl, ctypes.c_uint64), k,
                                  None, 0, ctypes.byref(need))
    if st != 0:
        raise RuntimeError(f"constraint compilation failed with status {st}")
    buf = ctypes.create_string_buffer(need.value)
    lib.pmo_dump_constraints(_p(po, ctypes.c_uint64), _p(pa, ctypes.c_uint32), _p(pl, ctypes.c_uint64), k, buf,
                             need.value, None)
    return buf.value.decode()
