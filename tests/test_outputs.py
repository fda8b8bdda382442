"""Output writers beyond results.totem: the match list and the pruned
subgraph.

- pm_query_list_matches lists the embeddings ENUMERATION counts, each as the
  vertices bound by the enumeration walk's vertex moves in walk order (the
  reference's writeEnumeration, multiple_label_enumeration_cpu.tpp:15-35,
  records historyIndexVector): the set of rows equals the oracle's listing,
  and their number equals the golden ENUMERATION count.
- pm_query_write_matches writes them in the reference's text form.
- pm_query_export_subgraph returns the CSR entries printActiveGraph prints
  (multiple_label_cpu.cc:270-284) as a CSR over the original ids.
"""
from __future__ import annotations

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from oracle import oracle
from tests import cases as C
from tests import pmtest

pytestmark = pytest.mark.gpu

SYNTH = {c["name"]: c for c in pmtest.load_synthetic_golden()}
NAMES = ["fixture3_s9", "triangle_rep_s9", "c1_scale10_cycle4", "k4_rep_s8", "two_cycles_s10", "path4_rep_s9",
         "random_12"]


def _sorted_rows(m: np.ndarray) -> list:
    return sorted(map(tuple, m.tolist()))


@pytest.mark.parametrize("name", NAMES)
def test_match_list_equals_oracle(name, tmp_path):
    case = SYNTH[name]
    g = C.make_graph(case)
    p = C.make_pattern(case)
    off, adj, lab = g.host_csr()
    want, n_want = oracle.list_matches(off, adj, lab, p.offsets, p.adj, p.labels, cap=case["rows"][-2][8])
    assert n_want == case["rows"][-2][8]
    q = pm.Query(g, pattern=p)
    got, n = q.list_matches(cap=n_want + 10)
    assert n == n_want
    assert got.shape == (n_want, p.n)
    assert _sorted_rows(got) == _sorted_rows(want)
    # The match list does not change the query: its full run is golden.
    assert [list(r.as_tuple()) for r in q.run()] == case["rows"]
    # Capped listing: the total is still reported.
    few, n2 = q.list_matches(cap=5)
    assert n2 == n_want and len(few) == min(5, n_want)
    assert set(map(tuple, few.tolist())) <= set(map(tuple, want.tolist()))
    path = tmp_path / "enumeration_0000.totem"
    assert q.write_matches(path, max_matches=n_want) == n_want
    lines = path.read_text().splitlines()
    assert sorted(lines) == sorted("".join(f"{x};" for x in r) for r in want.tolist())
    q.close()


def test_match_list_from_pattern_files():
    d = C.GOLDEN / "data" / "test_3"
    g = pm.Graph.load(d / "graph.totem", None, d / "vertex_data" / "graph_vertex_data.totem", device=0)
    q = pm.Query(g, pattern_dir=str(d / "pattern_1") + "/")
    m, n = q.list_matches()
    assert n == 2 and m.shape == (2, 4)
    q.close()


@pytest.mark.parametrize("name", ["fixture3_s9", "two_cycles_zipf_s10", "scale12_tds"])
def test_pruned_subgraph_equals_state(name):
    case = SYNTH[name]
    g = C.make_graph(case)
    q = pm.Query(g, pattern=C.make_pattern(case))
    q.run()
    cand, eact, vact = q.export()
    off, adj, _ = g.host_csr()
    s_off, s_adj = q.export_subgraph()
    V = g.vertex_count
    deg = np.diff(off.astype(np.int64))
    src = np.repeat(np.arange(V), deg)
    keep = (eact != 0) & (vact[src] != 0) & (vact[adj.astype(np.int64)] != 0)
    want_off = np.concatenate([[0], np.cumsum(np.bincount(src[keep], minlength=V))]).astype(np.uint64)
    assert np.array_equal(s_off, want_off)
    assert np.array_equal(s_adj, adj[keep])
    assert len(s_adj) > 0
    q.close()
