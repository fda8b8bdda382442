"""GPU parity: the sm_103a pipeline, called through the C ABI, against the
reference's own outputs (golden fixtures) and against the oracle.  Integer
work throughout, so every comparison is bit-exact: the results.totem rows
(timing columns excluded), the surviving (vertex, role) set (vertex_NNNN),
the active CSR entries (graph_NNNN) and the exact match count."""
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from oracle import oracle
from pattenmatching_sharedmemory_gb300 import templates as T
from tests import cases as C
from tests import pmtest

pytestmark = pytest.mark.gpu

FIXTURES = pmtest.load_fixture_golden()
SYNTH = pmtest.load_synthetic_golden()
DATA = pmtest.GOLDEN / "data"


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_fixture_outputs_identical(name):
    exp = FIXTURES[name]
    d = DATA / name
    g = pm.Graph.load(d / "graph.totem", None, d / "vertex_data" / "graph_vertex_data.totem", device=0)
    res = pmtest.product_run(g, pattern_dir=str(d / "pattern_1") + "/")
    assert res["rows"] == exp["rows"]
    assert res["last"] == exp["last"]
    assert res["vertex"].decode() == exp["vertex"]
    assert res["graph"].decode() == exp["graph"]


@pytest.mark.parametrize("case", SYNTH, ids=lambda c: c["name"])
def test_synthetic_outputs_identical(case):
    g = C.make_graph(case)
    res = pmtest.product_run(g, pattern=C.make_pattern(case))
    assert res["rows"] == case["rows"]
    assert pmtest.sha(res["vertex"]) == case["vertex_sha256"]
    assert pmtest.sha(res["graph"]) == case["graph_sha256"]


def _extra_cases():
    out = []
    for i in range(12):
        n = 3 + i % 6
        out.append({"name": f"extra_{i}", "graph": C.graph_params(9 + i % 2, ef=8, n_labels=2 + i % 3,
                                                                  label_seed=300 + i),
                    "pattern": {"kind": "random", "n": n, "density": 0.35 + 0.1 * (i % 3), "label_n": 2 + i % 3,
                                "zipf_s": 0.0, "seed": 9000 + i, "distinct": False}})
    return out


@pytest.mark.parametrize("case", _extra_cases(), ids=lambda c: c["name"])
def test_state_matches_oracle(case):
    """Cases outside the golden set, repeated labels (memo-heavy TDS/PC walks):
    every pruning step row and the final role sets and CSR-entry flags equal
    the oracle's (one thread, the canonical order).  The oracle stops before
    ENUMERATION here (these graphs have up to 2.5e10 matches, minutes of CPU);
    enumeration counts are pinned by the golden cases."""
    g = C.make_graph(case)
    p = C.make_pattern(case)
    off, adj, lab = g.host_csr()
    ref = oracle.run(off, adj, lab, p.offsets, p.adj, p.labels, threads=1, stop_before_enumeration=True)
    q = pm.Query(g, pattern=p)
    rows = [r.as_tuple() for r in q.prune()]
    # Both stop where the schedule would enter ENUMERATION; the last row names it.
    assert rows[-1][0] == "ENUMERATION"
    assert rows == ref.rows
    cand, eact, vact = q.export()
    assert np.array_equal(cand, ref.cand)
    assert np.array_equal(eact, ref.eact)
    assert np.array_equal(vact, ref.vact)


def test_step_api_equals_run():
    case = next(c for c in SYNTH if c["name"] == "fixture3_s9")
    g = C.make_graph(case)
    p = C.make_pattern(case)
    q1 = pm.Query(g, pattern=p)
    stepped = []
    while True:
        rec, fin = q1.step()
        stepped.append(rec.as_tuple())
        if fin:
            break
    q2 = pm.Query(g, pattern=p)
    ran = [r.as_tuple() for r in q2.run()]
    assert stepped == ran[:-1]
    assert ran[-1][0] == "END"


def test_cli_drop_in(tmp_path):
    """The CLI takes the reference's flags and writes the same files."""
    exp = FIXTURES["test_4"]
    d = DATA / "test_4"
    out = tmp_path / "out"
    subprocess.run([str(pm.CLI_PATH), "-i", str(d / "graph.totem"), "-b", str(tmp_path / "g.bin"), "-v",
                    str(d / "vertex_data" / "graph_vertex_data.totem"), "-p", str(d / "pattern_1") + "/", "-o",
                    str(out) + "/"], check=True, capture_output=True)
    rows = []
    for line in (out / "results.totem").read_text().splitlines()[1:]:
        f = [x.strip() for x in line.split(";")]
        rows.append([f[1]] + [int(x) for x in f[4:12]])
    assert rows == exp["rows"]
    assert (out / f"vertex_{exp['last']:04d}.totem").read_text() == exp["vertex"]
    assert (out / f"graph_{exp['last']:04d}.totem").read_text() == exp["graph"]
    assert (tmp_path / "g.bin").exists()


def test_queries_share_one_resident_graph():
    case = next(c for c in SYNTH if c["name"] == "two_cycles_s10")
    g = C.make_graph(case)
    a = pmtest.product_run(g, pattern=C.make_pattern(case))
    other = next(c for c in SYNTH if c["name"] == "c1_scale10_cycle4")
    g2 = C.make_graph(other)
    b = pmtest.product_run(g2, pattern=C.make_pattern(other))
    # same graph object, second template after the first
    c = pmtest.product_run(g, pattern=C.make_pattern(other)) if case["graph"] == other["graph"] else None
    assert a["rows"] == case["rows"] and b["rows"] == other["rows"]
    if c is not None:
        assert c["rows"] == other["rows"]


# LCC degree classes: (hub_degree, seg_entries).  (0, 32) makes every vertex
# with an edge a hub, most of them with several 32-entry segments; the others
# mix light tiles with multi-segment hubs.  The plan changes speed only.
HUB_PLANS = [(0, 32), (4, 32), (16, 64), (64, 128), (8, 1024)]
HUB_PLAN_CASES = ["scale12_tds", "two_cycles_zipf_s10", "path4_rep_s9", "degree_labels_s10"]


@pytest.mark.parametrize("plan", HUB_PLANS, ids=lambda p: f"h{p[0]}_s{p[1]}")
@pytest.mark.parametrize("name", HUB_PLAN_CASES)
def test_hub_plan_outputs_identical(name, plan):
    case = next(c for c in SYNTH if c["name"] == name)
    g = C.make_graph(case).to_device(0)
    g.set_hub_plan(*plan)
    res = pmtest.product_run(g, pattern=C.make_pattern(case))
    assert res["rows"] == case["rows"]
    assert pmtest.sha(res["vertex"]) == case["vertex_sha256"]
    assert pmtest.sha(res["graph"]) == case["graph_sha256"]


@pytest.mark.parametrize("plan", [None, (4, 32)], ids=["default", "h4_s32"])
def test_many_needed_slots_matches_oracle(plan):
    """A 17-leaf star with distinct labels needs 17 label slots counted per
    vertex: more than the per-owner counters, so light tiles and hubs take the
    whole-list warp path.  Pruning rows and the final state equal the
    oracle's."""
    g = C.make_graph({"graph": C.graph_params(10, ef=16, n_labels=20, label_seed=77)}).to_device(0)
    if plan:
        g.set_hub_plan(*plan)
    p = pm.Pattern.from_edges(18, [(0, i) for i in range(1, 18)], list(range(18)))
    off, adj, lab = g.host_csr()
    ref = oracle.run(off, adj, lab, p.offsets, p.adj, p.labels, threads=1, stop_before_enumeration=True)
    q = pm.Query(g, pattern=p)
    rows = [r.as_tuple() for r in q.run()]
    assert rows[:-2] == ref.rows[:-1]
    cand, eact, vact = q.export()
    assert np.array_equal(cand, ref.cand)
    assert np.array_equal(eact, ref.eact)
    assert np.array_equal(vact, ref.vact)


def test_hub_plan_change_with_live_query():
    """A plan that adds hubs after a query was created: the query's hub
    accumulators grow before its next step and results stay exact."""
    case = next(c for c in SYNTH if c["name"] == "scale12_tds")
    g = C.make_graph(case).to_device(0)
    g.set_hub_plan(1 << 26, 1024)  # no hubs
    q = pm.Query(g, pattern=C.make_pattern(case))
    first, fin = q.step()
    g.set_hub_plan(2, 32)
    rows = [list(first.as_tuple())]
    while not fin:
        rec, fin = q.step()
        rows.append(list(rec.as_tuple()))
    assert rows == case["rows"][:-1]


# Speed knobs at extreme settings: 1-entry first-hop slices for walks and
# enumeration (every source split), the smallest memo tables (overflow
# re-runs and table growth), and no slicing at all.  Results must not move.
KNOB_SETTINGS = {
    "slice_everything": {"walk_presplit": 1, "enum_presplit": (1, 1), "walk_tables": 1024, "enum_tables": 1024},
    "no_slicing": {"walk_presplit": 0, "enum_presplit": (0, 0), "walk_tables": 1024, "enum_tables": 1024},
    "split_on_overflow_only": {"walk_presplit": 0, "enum_presplit": (0, 0), "walk_tables": 2048,
                               "enum_tables": 1024, "enum_split": (2, 0)},
    # ENUMERATION tail from the source's side whenever the source is cached,
    # and never.
    "tail_swap_always": {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192, "enum_tables": 8192,
                         "tail_swap": 1, "walk_tail_swap": 1},
    "tail_swap_off": {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192, "enum_tables": 8192,
                      "tail_swap": 0, "walk_tail_swap": 0},
    # The step before the tail one candidate at a time (pair-parallel off),
    # and pair-parallel with the source-side tail off.
    "pair_tail_off": {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192, "enum_tables": 8192,
                      "pair_tail": (0, 0)},
    "pair_tail_no_swap": {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192, "enum_tables": 8192,
                          "pair_tail": (1, 1), "tail_swap": 0, "walk_tail_swap": 0},
    # Second-hop slices everywhere they apply (every source sliced, 4-entry
    # second-hop slices of lists above 8 entries), with and without the pair
    # step, and never.
    "second_split_small": {"walk_presplit": 64, "enum_presplit": (1, 1), "walk_tables": 8192, "enum_tables": 8192,
                           "second_split": 4},
    "second_split_small_no_pair": {"walk_presplit": 64, "enum_presplit": (2, 2), "walk_tables": 8192,
                                   "enum_tables": 8192, "second_split": 4, "pair_tail": (0, 0)},
    "second_split_off": {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192, "enum_tables": 8192,
                         "second_split": 0},
    # ENUMERATION without the count memo (every subtree walked).
    "count_memo_off": {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192, "enum_tables": 8192,
                       "count_memo": 0},
    # Exact CC/PC/TDS without the state memo before the tail, with and
    # without the swapped tail.
    "walk_tail_no_state_memo": {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192,
                                "enum_tables": 8192, "tail_state_memo": 0},
    "walk_tail_no_state_memo_no_swap": {"walk_presplit": 0, "enum_presplit": (32, 8), "walk_tables": 8192,
                                        "enum_tables": 8192, "tail_state_memo": 0, "walk_tail_swap": 0},
    # Exact CC/PC/TDS slices (first-hop slices of every item) with the
    # swapped tail on every cached source.
    "walk_slices_tail_swap": {"walk_presplit": 1, "enum_presplit": (32, 8), "walk_tables": 8192,
                              "enum_tables": 8192, "walk_tail_swap": 1},
}
KNOB_CASES = ["scale12_tds", "cycle5_s10", "path4_rep_s9", "two_cycles_zipf_s10", "random_08", "k4_rep_s8",
              "c1_scale10_cycle4"]


def _set_knobs(k):
    pm.lib.pm_set_walk_presplit(k["walk_presplit"])
    pm.lib.pm_set_enum_presplit_by_kind(*k["enum_presplit"])
    pm.lib.pm_set_walk_table_entries(k["walk_tables"])
    pm.lib.pm_set_enum_table_entries(k["enum_tables"])
    pm.lib.pm_set_enum_split(*k.get("enum_split", (16, 0)))
    pm.lib.pm_set_enum_tail_swap(k.get("tail_swap", 4))
    pm.lib.pm_set_walk_tail_swap(k.get("walk_tail_swap", 4))
    pm.lib.pm_set_enum_count_memo(k.get("count_memo", 1))
    pm.lib.pm_set_walk_tail_state_memo(k.get("tail_state_memo", 1))
    pm.lib.pm_set_pair_tail(*k.get("pair_tail", (1, 1)))
    pm.lib.pm_set_enum_second_split(k.get("second_split", 256))


DEFAULT_KNOBS = {"walk_presplit": 64, "enum_presplit": (32, 8), "walk_tables": 8192, "enum_tables": 8192,
                 "enum_split": (16, 0)}


@pytest.mark.parametrize("setting", sorted(KNOB_SETTINGS))
@pytest.mark.parametrize("name", KNOB_CASES)
def test_knob_settings_outputs_identical(name, setting):
    case = next(c for c in SYNTH if c["name"] == name)
    g = C.make_graph(case).to_device(0)
    _set_knobs(KNOB_SETTINGS[setting])
    try:
        res = pmtest.product_run(g, pattern=C.make_pattern(case))
    finally:
        _set_knobs(DEFAULT_KNOBS)
    assert res["rows"] == case["rows"]
    assert pmtest.sha(res["vertex"]) == case["vertex_sha256"]
    assert pmtest.sha(res["graph"]) == case["graph_sha256"]


LCC_GRAPH_CASES = ["scale12_tds", "cycle5_s10", "two_cycles_zipf_s10", "random_08", "fixture3_s9",
                   "c1_scale10_cycle4", "k4_rep_s8"]


def _rows_and_state(g, p):
    q = pm.Query(g, pattern=p)
    recs = q.run()
    rows = [r.as_tuple() for r in recs]
    cand, eact, vact = q.export()
    count = q.match_count
    q.close()
    return recs, rows, count, cand, eact, vact


@pytest.mark.parametrize("name", LCC_GRAPH_CASES)
def test_lcc_graph_equals_host_loop(name):
    """Each LCC fixpoint as one CUDA-graph launch (a conditional WHILE node
    whose tail kernel records the pass and decides on the device whether
    another pass runs) gives the rows, count and state of the host-driven
    loop (one launch sequence and counter read-back per pass)."""
    case = next(c for c in SYNTH if c["name"] == name)
    g = C.make_graph(case).to_device(0)
    p = C.make_pattern(case)
    pm._check(pm.lib.pm_set_lcc_graph(0))
    try:
        host = _rows_and_state(g, p)
    finally:
        pm._check(pm.lib.pm_set_lcc_graph(1))
    graph = _rows_and_state(g, p)
    assert graph[1] == host[1]
    assert graph[1] == [tuple(r) for r in case["rows"]]
    assert graph[2] == host[2]
    for a, b in zip(graph[3:], host[3:]):
        assert np.array_equal(a, b)
    lcc = [r for r in graph[0] if r.as_tuple()[0] == "LCC"]
    assert lcc and all(r.step_ms >= 0 for r in lcc)
    cum = [r.cumulative_ms for r in graph[0]]
    assert cum == sorted(cum)


@pytest.mark.parametrize("name", LCC_GRAPH_CASES)
def test_lcc_label_stream_equals_gather(name):
    """The first LCC pass after LCC0 from the entry label bytes gives the
    rows, count and state of the pass that gathers neighbour words, through
    the captured loop and the host-driven loop alike."""
    case = next(c for c in SYNTH if c["name"] == name)
    g = C.make_graph(case).to_device(0)
    p = C.make_pattern(case)
    pm._check(pm.lib.pm_set_lcc_label_stream(0))
    try:
        gather = _rows_and_state(g, p)
    finally:
        pm._check(pm.lib.pm_set_lcc_label_stream(1))
    for graph_loop in (1, 0):
        pm._check(pm.lib.pm_set_lcc_graph(graph_loop))
        try:
            label = _rows_and_state(g, p)
        finally:
            pm._check(pm.lib.pm_set_lcc_graph(1))
        assert label[1] == gather[1] == [tuple(r) for r in case["rows"]]
        assert label[2] == gather[2]
        for a, b in zip(label[3:], gather[3:]):
            assert np.array_equal(a, b)
    # The first LCC row read no neighbour word; the gathering run's did.
    first_lcc = next(i for i, r in enumerate(gather[1]) if r[0] == "LCC")
    q = pm.Query(g, pattern=p)
    q.step()
    q.step()
    assert q.step_walk_stats(first_lcc)[1] == 0
    q.close()
    g.close()


def test_lcc_graph_follows_hub_plan_change():
    """A plan change between queries rebuilds the captured loop (its kernels
    bake the graph's segment table)."""
    case = next(c for c in SYNTH if c["name"] == "scale12_tds")
    g = C.make_graph(case).to_device(0)
    p = C.make_pattern(case)
    try:
        for plan in [(16, 64), (32, 1024), (8, 32)]:
            g.set_hub_plan(*plan)
            rows = _rows_and_state(g, p)[1]
            assert rows == [tuple(r) for r in case["rows"]], plan
    finally:
        g.set_hub_plan(32, 1024)


def test_lcc_graph_alternating_graphs_one_thread():
    """One host thread alternating between two resident graphs (and word
    types) reuses a captured loop per graph: every run still gives the
    golden rows."""
    cases = [next(c for c in SYNTH if c["name"] == n) for n in ("scale12_tds", "k4_rep_s8")]
    graphs = [C.make_graph(c).to_device(0) for c in cases]
    for _ in range(2):
        for c, g in zip(cases, graphs):
            rows = _rows_and_state(g, C.make_pattern(c))[1]
            assert rows == [tuple(r) for r in c["rows"]], c["name"]


@pytest.mark.parametrize("name,rescues,overflows", [("random_10", 1, 1), ("random_11", 1, 1), ("random_15", 1, 1),
                                                     ("k4_rep_s8", 0, 1), ("random_03", 1, 0)])
def test_rescue_replay_and_overflow_reruns_run(name, rescues, overflows):
    """Golden cases that reach the two rare paths: the host replay of the
    reference's alreadyMatched shortcut (a failing walk that an earlier
    success marked, multiple_label_cc_cpu.tpp:107) and the re-run of walks
    whose memo tables overflowed.  The statistics prove the paths ran; the
    rows prove they kept the reference's results."""
    case = next(c for c in SYNTH if c["name"] == name)
    g = C.make_graph(case)
    q = pm.Query(g, pattern=C.make_pattern(case))
    rows = [list(r.as_tuple()) for r in q.run()]
    st = q.stats()
    q.close()
    assert rows == case["rows"]
    assert st["exact_resolutions"] >= rescues
    assert st["overflow_retries"] >= overflows
