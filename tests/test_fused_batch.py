"""The batched form (pm_fused_batch_*): many templates in lockstep rounds,
their LCC0 steps and LCC fixpoints in shared multi-query launches.

Contract: every query's rows (timing columns aside), match count and final
state (role sets, CSR-entry and vertex flags) equal the same template run
alone through pm_query_run, bit for bit, since all of it is integer work;
with PM_SUBMIT_PRUNE_ONLY they equal pm_query_prune's.  The batch mixes
word types (templates of up to 8, 24 and 56 vertices), repeated and
distinct labels, CC / PC / TDS schedules and templates whose state empties.
"""
from __future__ import annotations

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from pattenmatching_sharedmemory_gb300 import templates as T
from tests import cases as C
from tests import pmtest

pytestmark = pytest.mark.gpu

SYNTH = {c["name"]: c for c in pmtest.load_synthetic_golden()}
MIX = ["c1_scale10_cycle4", "triangle_rep_s9", "path4_rep_s9", "fixture3_s9", "k4_rep_s8", "two_cycles_s10",
       "scale12_tds", "cycle4_rep_s9", "star_s9", "fixture1_s10_zipf", "path_rep_s9", "cycle5_s10"]


def _patterns():
    ps = [C.make_pattern(SYNTH[n]) for n in MIX]
    # wider word types: a 12-vertex template (32-bit words: a 4-cycle and a
    # tail of 8) and a 26-vertex path (64-bit words), each with distinct
    # labels of which the last ones no vertex carries, so their roles fall
    # one layer per LCC pass until the state is empty.  (Templates of that
    # size with repeated labels make template-driven searches that run for
    # minutes on this graph, in the reference's walks and on the GPU alike.)
    ps.append(pm.Pattern.from_edges(12, [(0, 1), (1, 2), (2, 3), (3, 0)] + [(i, i + 1) for i in range(3, 11)],
                                    list(range(8)) + [20, 21, 22, 23]))
    ps.append(pm.Pattern.from_edges(26, [(i, i + 1) for i in range(25)], list(range(8)) + list(range(20, 38))))
    # a template whose labels no vertex carries: the state empties at LCC0
    ps.append(T.cycle([50, 51, 52]))
    return ps


def _alone(g, p, prune_only):
    q = pm.Query(g, pattern=p)
    recs = q.prune() if prune_only else q.run()
    rows = [r.as_tuple() for r in recs]
    cand, eact, vact = q.export()
    count = q.match_count
    q.close()
    return rows, count, cand, eact, vact


@pytest.mark.parametrize("prune_only", [False, True])
def test_fused_batch_equals_alone(prune_only):
    g = C.make_graph(SYNTH["scale12_tds"]).to_device(0)
    ps = _patterns()
    alone = [_alone(g, p, prune_only) for p in ps]
    with pm.FusedBatch(g, ps, prune_only=prune_only) as b:
        st = b.stats()
        assert st["shared_lcc_phases"] > 0 and st["rounds"] > 1
        for i, p in enumerate(ps):
            r = b.result(i)
            assert r.status == pm.PM_SUCCESS, (i, r.status)
            rows, count, cand, eact, vact = alone[i]
            assert [x.as_tuple() for x in b.records(i)] == rows, i
            assert r.match_count == count
            c2, e2, v2 = b.export(i)
            assert np.array_equal(c2, cand) and np.array_equal(e2, eact) and np.array_equal(v2, vact), i
    g.close()


def test_fused_batch_golden_rows():
    """The golden synthetic cases that share one graph, batched: the
    reference's own rows."""
    by_graph = {}
    for c in SYNTH.values():
        if c.get("big"):
            continue
        by_graph.setdefault(repr(c["graph"]), []).append(c)
    key, cases = max(by_graph.items(), key=lambda kv: len(kv[1]))
    g = C.make_graph(cases[0]).to_device(0)
    with pm.FusedBatch(g, [C.make_pattern(c) for c in cases]) as b:
        for i, c in enumerate(cases):
            assert b.result(i).status == pm.PM_SUCCESS
            assert [list(x.as_tuple()) for x in b.records(i)] == c["rows"], c["name"]
    g.close()


def test_fused_batch_budget_ends_slow_queries_only():
    """With a per-query budget the slow query times out while the others
    keep their exact results."""
    big = SYNTH["c1_scale16_cycle4"]
    g = C.make_graph(big).to_device(0)
    slow = C.make_pattern(big)
    fast = [T.cycle([0, 1, 2]), T.cycle([4, 4, 3])]
    alone = [_alone(g, p, True) for p in fast]
    assert pm.lib.pm_set_query_budget_ms(3.0) == pm.PM_SUCCESS
    try:
        with pm.FusedBatch(g, [slow] + fast, prune_only=False) as b:
            assert b.result(0).status == pm.PM_E_TIMEOUT
    finally:
        pm.lib.pm_set_query_budget_ms(0.0)
    with pm.FusedBatch(g, [slow] + fast, prune_only=True) as b:
        for i, p in enumerate(fast):
            assert [x.as_tuple() for x in b.records(i + 1)] == alone[i][0]
    g.close()
