"""pm_enumerate_noalloc: the allocation-free ENUMERATION entry point.

It counts embeddings over a pruned state the caller holds on the device,
using only the library's fixed __device__ scratch array.  Its count must equal
the one the regular pipeline (pm_query_run -> ENUMERATION row) reports for the
same state, bit for bit, on consecutive calls: the array keeps the previous
call's contents, so a second call checks that everything that must start at
zero is cleared.  This file is collected last so that it runs both alone in a
fresh process and after every other test in one session.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from pattenmatching_sharedmemory_gb300 import templates as T

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 26


def _dev(a: np.ndarray):
    import torch

    signed = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32}[a.dtype]
    return torch.from_numpy(np.ascontiguousarray(a).view(signed)).to("cuda:0")


def _edge_bits(eact: np.ndarray) -> np.ndarray:
    """Per-CSR-entry flags -> one bit per entry, bit e % 32 of word e // 32."""
    b = np.packbits(eact.astype(np.uint8) != 0, bitorder="little")
    buf = np.zeros(max((len(eact) + 31) // 32, 1) * 4, np.uint8)
    buf[:len(b)] = b
    return buf.view("<u4").astype(np.uint32)


def _sorted_unique(off: np.ndarray, adj: np.ndarray) -> int:
    d = np.diff(adj.astype(np.int64))
    inside = np.ones(len(d), bool)
    starts = off[1:-1].astype(np.int64) - 1  # last pair index of each row
    starts = starts[(starts >= 0) & (starts < len(d))]
    inside[starts] = False
    return int(bool(np.all(d[inside] > 0)))


class _State:
    """A graph and one template's pruned state, uploaded for the entry point."""

    def __init__(self, g: pm.Graph, tmpl: pm.Pattern):
        q = pm.Query(g, pattern=tmpl)
        q.run()
        self.expected = q.match_count
        cand, eact, _ = q.export()
        q.close()
        off, adj, _ = g.host_csr()
        self.V, self.E = g.vertex_count, g.edge_count
        self.sorted_unique = _sorted_unique(off, adj)
        self.d_off, self.d_adj = _dev(off.copy()), _dev(adj.copy() if len(adj) else np.zeros(1, np.uint32))
        self.d_cand = _dev(cand)
        self.d_eact = _dev(_edge_bits(eact))
        self.p_off = np.ascontiguousarray(tmpl.offsets, np.uint64)
        self.p_adj = np.ascontiguousarray(tmpl.adj, np.uint32)
        self.p_lab = np.ascontiguousarray(tmpl.labels, np.uint64)

    def call(self, d_count, *, vertex_count=None, p_vertex_count=None) -> int:
        return pm.lib.pm_enumerate_noalloc(
            self.d_off.data_ptr(), self.d_adj.data_ptr(), self.V if vertex_count is None else vertex_count, self.E,
            self.sorted_unique, self.d_cand.data_ptr(), self.d_eact.data_ptr(),
            self.p_off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            self.p_adj.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
            self.p_lab.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            len(self.p_off) - 1 if p_vertex_count is None else p_vertex_count, len(self.p_adj),
            d_count.data_ptr(), None)


@pytest.fixture(scope="module")
def states():
    g = pm.Graph.rmat(12, 16, seed=3).assign_labels("uniform", 5, 1.0, 2).to_device(0)
    n, edges, labels = (4, [(0, 1), (0, 2), (0, 3), (1, 2), (2, 3)], [0, 1, 2, 1])
    out = {
        "cycle4_distinct": _State(g, T.cycle([0, 1, 2, 3])),
        "cycle5_distinct": _State(g, T.cycle([0, 1, 2, 3, 4])),
        "diamond_repeated": _State(g, pm.Pattern.from_edges(n, edges, labels)),
    }
    yield out
    g.close()


def _count(st: _State, d_count) -> int:
    d_count.fill_(-1)
    status = st.call(d_count)
    assert status == pm.PM_SUCCESS, pm.lib.pm_last_error().decode()
    return int(d_count.item())


@pytest.mark.parametrize("name", ["cycle4_distinct", "cycle5_distinct", "diamond_repeated"])
def test_noalloc_matches_pipeline_twice(states, name):
    import torch

    st = states[name]
    assert st.expected > 0
    d_count = torch.empty(1, dtype=torch.int64, device="cuda:0")
    first = _count(st, d_count)
    second = _count(st, d_count)
    # Integer counts: bit-exact against the regular entry point, both calls.
    assert first == st.expected
    assert second == st.expected


def test_noalloc_interleaved_templates(states):
    import torch

    d_count = torch.empty(1, dtype=torch.int64, device="cuda:0")
    order = ["cycle5_distinct", "diamond_repeated", "cycle4_distinct", "cycle5_distinct"]
    got = [_count(states[n], d_count) for n in order]
    assert got == [states[n].expected for n in order]


def test_noalloc_rejects_beyond_limits(states):
    import torch

    st = states["cycle4_distinct"]
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    status = st.call(d_count, vertex_count=MAX_VERTICES + 1)
    assert status == pm.PM_E_INVALID_ARG
    assert "67108864" in pm.lib.pm_last_error().decode()
    big = T.cycle(list(range(57)))
    st2 = object.__new__(_State)
    st2.__dict__.update(st.__dict__)
    st2.p_off = np.ascontiguousarray(big.offsets, np.uint64)
    st2.p_adj = np.ascontiguousarray(big.adj, np.uint32)
    st2.p_lab = np.ascontiguousarray(big.labels, np.uint64)
    assert st2.call(d_count) == pm.PM_E_PATTERN_TOO_LARGE
    assert int(d_count.item()) == 0


def test_noalloc_retry_rounds(states):
    """Tiny first-round tables make sources overflow, so later rounds re-run
    them from the bitmap of overflowed sources with 4x larger tables (and
    the two bitmaps swap roles between rounds); the count must not change."""
    import torch

    d_count = torch.empty(1, dtype=torch.int64, device="cuda:0")
    assert pm.lib.pm_set_noalloc_table_entries(32) == pm.PM_SUCCESS
    try:
        for name in ("cycle5_distinct", "cycle4_distinct", "cycle5_distinct"):
            assert _count(states[name], d_count) == states[name].expected
            assert pm.lib.pm_noalloc_last_rounds() >= 2, name
    finally:
        assert pm.lib.pm_set_noalloc_table_entries(2048) == pm.PM_SUCCESS
    assert _count(states["cycle4_distinct"], d_count) == states["cycle4_distinct"].expected
    assert pm.lib.pm_noalloc_last_rounds() == 1
    assert pm.lib.pm_set_noalloc_table_entries(48) == pm.PM_E_INVALID_ARG
