"""The served RMAT-16 stream's 15 templates (every 4-subset of labels 0..4 in
its 3 cyclic orders, 4-cycles with distinct labels), full pipeline with exact
ENUMERATION (6.5e7-7.2e7 matches each), pinned against the reference's own
outputs: every row (timing columns aside), the surviving role sets and the
active CSR entries, as the golden file holds them.

The golden runs took the reference about a quarter of an hour each on five
threads; with distinct template labels no memo test can block a walk, so
their outputs do not depend on the thread count.  The 0-1-2-3 cycle is also
the one-thread golden case c1_scale16_cycle4: both must agree.
"""
from __future__ import annotations

import json

import pytest

import pattenmatching_sharedmemory_gb300 as pm
from tests import cases as C
from tests import pmtest

GOLDEN = pmtest.GOLDEN / "stream15_rmat16.json"
STREAM = json.loads(GOLDEN.read_text()) if GOLDEN.exists() else []
NAMES = {c["name"]: c for c in C.stream15_cases()}


def test_stream15_golden_describes_the_stream():
    assert STREAM, "no stream15 golden entries"
    seen = set()
    for e in STREAM:
        spec = NAMES[e["name"]]
        assert e["name"] not in seen
        seen.add(e["name"])
        assert e["pattern"] == spec["pattern"] and e["graph"] == spec["graph"]
        assert e["rows"][-1][0] == "END" and e["rows"][-2][0] == "ENUMERATION"
        assert e["rows"][-2][8] > 0


def test_stream15_thread_count_independent():
    """The 0-1-2-3 cycle: the five-thread stream run and the one-thread
    golden case give the same rows."""
    by_name = {e["name"]: e for e in STREAM}
    one = {c["name"]: c for c in pmtest.load_synthetic_golden()}.get("c1_scale16_cycle4")
    if "stream15_0123" not in by_name or one is None:
        pytest.skip("stream15_0123 or c1_scale16_cycle4 not in the golden files")
    five = by_name["stream15_0123"]
    assert one["ref_threads"] == 1 and five["ref_threads"] > 1
    assert one["rows"] == five["rows"]
    assert one["vertex_sha256"] == five["vertex_sha256"] and one["graph_sha256"] == five["graph_sha256"]


@pytest.fixture(scope="module")
def stream_graph():
    g = C.make_graph(NAMES["stream15_0123"]).to_device(0)
    yield g
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("entry", STREAM, ids=lambda e: e["name"])
def test_stream15_outputs_identical(entry, stream_graph):
    res = pmtest.product_run(stream_graph, pattern=C.make_pattern(entry))
    assert res["rows"] == entry["rows"]
    assert pmtest.sha(res["vertex"]) == entry["vertex_sha256"]
    assert pmtest.sha(res["graph"]) == entry["graph_sha256"]
    res["query"].close()


@pytest.mark.gpu
def test_stream15_served_counts(stream_graph):
    """The same templates through the server, all at once: each request's
    match count is its golden count."""
    with pm.Server(stream_graph, slots=8) as srv:
        tickets = [srv.submit(C.make_pattern(e), prune_only=False) for e in STREAM]
        for e, t in zip(STREAM, tickets):
            r = srv.wait(t)
            assert r.status == pm.PM_SUCCESS, e["name"]
            assert r.match_count == e["rows"][-2][8], e["name"]
