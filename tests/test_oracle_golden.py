"""The oracle (CPU restatement) pinned against the reference's own outputs.

The golden vectors come from the reference's compiled CPU path run with one
thread (tests/golden/make_golden.py): its bundled fixtures
data/patternmatching/test_{1..4} and seeded synthetic RMAT cases."""
import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from oracle import oracle
from tests import cases as C
from tests import pmtest

FIXTURES = pmtest.load_fixture_golden()
SYNTH = pmtest.load_synthetic_golden()


def _fixture_inputs(name):
    d = pmtest.GOLDEN / "data" / name
    g = pm.Graph.load(d / "graph.totem", None, d / "vertex_data" / "graph_vertex_data.totem", device=-1)
    pg = pm.Graph.load(d / "pattern_1" / "pattern_edge", None, d / "pattern_1" / "pattern_vertex_data", device=-1)
    return g, pg


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_oracle_matches_reference_fixture(name):
    exp = FIXTURES[name]
    g, pg = _fixture_inputs(name)
    off, adj, lab = g.host_csr()
    po, pa, pl = pg.host_csr()
    r = oracle.run(off, adj, lab, po, pa, pl)
    assert [list(x) for x in r.rows] == exp["rows"]
    assert pmtest.vertex_text(r.cand, r.vact).decode() == exp["vertex"]
    assert pmtest.graph_text(off, adj, lab, r.eact, r.vact).decode() == exp["graph"]


def _small(case):
    # Keep the CPU suite to a few minutes: the oracle enumerates every match.
    return case["rows"][-2][8] <= 4_000_000 and not case.get("big")


@pytest.mark.parametrize("case", [c for c in SYNTH if _small(c)], ids=lambda c: c["name"])
def test_oracle_matches_reference_synthetic(case):
    g, r = pmtest.oracle_case(case)
    off, adj, lab = g.host_csr()
    assert [list(x) for x in r.rows] == case["rows"]
    assert pmtest.sha(pmtest.vertex_text(r.cand, r.vact)) == case["vertex_sha256"]
    assert pmtest.sha(pmtest.graph_text(off, adj, lab, r.eact, r.vact)) == case["graph_sha256"]


def test_oracle_threads_agree_on_distinct_labels():
    # With distinct-label templates the walks have no memo false negatives,
    # so the thread count cannot change the result.
    case = next(c for c in SYNTH if c["name"] == "c1_scale10_cycle4")
    _, r1 = pmtest.oracle_case(case, threads=1)
    _, r4 = pmtest.oracle_case(case, threads=4)
    assert r1.rows == r4.rows
    assert np.array_equal(r1.cand, r4.cand) and np.array_equal(r1.eact, r4.eact)
