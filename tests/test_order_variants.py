"""The article's constraint-order drivers (test_article/CMakeLists.txt:53-73):
backtrack walks with all three optimisations, every NLCC constraint run once
and dropped, and either the fixed cycle / path / template order ending in
ENUMERATION (order_enumerate_intuitive) or the dynamic order
(ORDER_USE_DYNAMIC): after every LCC fixpoint the graph statistics of the
pruned graph are taken and the remaining constraint with the largest
estimated effectiveness runs next (test_order_multiple_label_cpu.cc:177-300),
optionally starting ENUMERATION early (ENUMERATE_START_EARLY, threshold 0.01).

Golden vectors: the reference's own order binaries
(oracle/_ref/patternmatching_order_*, `make -C oracle ref-order`) on the
bundled fixtures and the seeded synthetic cases, with one thread and, for
some cases, three (tests/golden/make_golden.py --only order).  The CPU test
pins the oracle restatement (its own graph-statistics loop) to them; the GPU
tests run the product (graph statistics on the device) against them, rows and
final state.  With several threads the reference's alreadyMatched shortcut
depends on timing, so multi-thread entries are compared only for templates
whose labels are pairwise distinct (the shortcut cannot change an outcome
then)."""
from __future__ import annotations

import json

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from oracle import oracle
from tests import cases as C
from tests import pmtest

GOLDEN = json.loads((pmtest.GOLDEN / "order_variants.json").read_text())
BACKTRACK = 2


def _inputs(entry):
    if entry["fixture"]:
        d = pmtest.GOLDEN / "data" / entry["fixture"]
        g = pm.Graph.load(d / "graph.totem", None, d / "vertex_data" / "graph_vertex_data.totem", device=-1)
        pg = pm.Graph.load(d / "pattern_1" / "pattern_edge", None, d / "pattern_1" / "pattern_vertex_data",
                           device=-1)
        po, pa, pl = pg.host_csr()
        return g, pm.Pattern(po.copy(), pa.copy(), pl.copy())
    return C.make_graph(entry["case"]), C.make_pattern(entry["case"])


def _comparable(entry) -> bool:
    if entry["aborted"]:
        return False
    if entry["threads"] == 1:
        return True
    _, p = _inputs(entry)
    return len(set(np.asarray(p.labels).tolist())) == p.n


def _check(entry, rows, cand, eact, vact, g):
    off, adj, lab = g.host_csr()
    assert [list(x) for x in rows] == entry["rows"]
    assert pmtest.sha(pmtest.vertex_text(cand, vact)) == entry["vertex_sha256"]
    assert pmtest.sha(pmtest.graph_text(off, adj, lab, eact, vact)) == entry["graph_sha256"]


ENTRIES = [e for e in GOLDEN if _comparable(e)]
# Cases whose backtrack walks take the CPU restatement seconds to minutes
# (the reference's own binaries too); the GPU test still covers them.
SLOW_ON_CPU = {"random_04", "random_05", "random_11"}


def _id(e):
    return f"{e['name']}-{e['order']}-t{e['threads']}"


def test_golden_covers_every_order_driver():
    assert {e["order"] for e in ENTRIES} == {"enumerate_intuitive", "effectiveness", "enumerate_effectiveness",
                                             "enumerate_effectiveness_early"}
    assert any(e["threads"] > 1 for e in ENTRIES)
    # The dynamic order really reorders: some case's effectiveness rows differ
    # from its fixed-order rows beyond the first (START) row and LCC0.
    by = {(e["name"], e["order"], e["threads"]): e for e in ENTRIES}
    differs = 0
    for (name, order, t), e in by.items():
        if order != "enumerate_effectiveness" or (name, "enumerate_intuitive", t) not in by:
            continue
        fixed = [r for r in by[(name, "enumerate_intuitive", t)]["rows"] if r[0] in ("CC", "PC", "TDS")]
        dyn = [r for r in e["rows"] if r[0] in ("CC", "PC", "TDS")]
        differs += fixed != dyn
    assert differs > 0


@pytest.mark.parametrize("entry", [e for e in ENTRIES if e["name"] not in SLOW_ON_CPU], ids=_id)
def test_oracle_order_matches_reference(entry):
    g, p = _inputs(entry)
    off, adj, lab = g.host_csr()
    r = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, variant=BACKTRACK,
                      order=pm.ORDER_DRIVERS[entry["order"]], order_threads=entry["threads"])
    _check(entry, r.rows, r.cand, r.eact, r.vact, g)


def test_order_flags_need_an_article_variant():
    g = pm.Graph.rmat(6, 4, seed=1).assign_labels("uniform", 3, seed=1)
    p = pm.Pattern.from_edges(3, [(0, 1), (1, 2), (2, 0)], [0, 1, 2])
    with pytest.raises(pm.PmError) as e:
        pm.Query(g, pattern=p, order="effectiveness")  # reference walks + order flags
    assert e.value.code == pm.PM_E_INVALID_ARG
    with pytest.raises(pm.PmError) as e:
        pm.Query(g, pattern=p, variant="backtrack", order=pm.PM_ORDER_EARLY_ENUMERATION)
    assert e.value.code == pm.PM_E_INVALID_ARG
    with pytest.raises(pm.PmError):
        pm.set_order_threads(0)


@pytest.mark.gpu
@pytest.mark.parametrize("entry", ENTRIES, ids=_id)
def test_gpu_order_matches_reference(entry):
    g, p = _inputs(entry)
    g.to_device(0)
    pm.set_order_threads(entry["threads"])
    try:
        q = pm.Query(g, pattern=p, variant="backtrack", order=entry["order"])
    finally:
        pm.set_order_threads(1)
    rows = [r.as_tuple() for r in q.run()]
    cand, eact, vact = q.export()
    q.close()
    _check(entry, rows, cand, eact, vact, g)


DISTINCT = [c for c in C.synthetic_cases(include_big=False)
            if len(set(C.make_pattern(c).labels.tolist())) == C.make_pattern(c).n][:6]


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [7, 60])
@pytest.mark.parametrize("case", DISTINCT, ids=lambda c: c["name"])
def test_gpu_dynamic_order_partitions_equal_oracle(case, threads):
    """The graph statistics' per-block accumulation under other thread
    counts (the reference's default is 60): device blocks against the
    oracle's sequential per-block loop, through the whole dynamic run."""
    g, p = C.make_graph(case), C.make_pattern(case)
    off, adj, lab = g.host_csr()
    flags = pm.ORDER_DRIVERS["enumerate_effectiveness_early"]
    try:
        ref = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, variant=BACKTRACK, order=flags,
                            order_threads=threads)
    except oracle.StatMissing:
        ref = None
    g.to_device(0)
    pm.set_order_threads(threads)
    try:
        q = pm.Query(g, pattern=p, variant="backtrack", order=flags)
    finally:
        pm.set_order_threads(1)
    if ref is None:
        with pytest.raises(pm.PmError) as e:
            q.run()
        assert e.value.code == pm.PM_E_STATISTICS
        q.close()
        return
    rows = [r.as_tuple() for r in q.run()]
    cand, eact, vact = q.export()
    q.close()
    assert rows == ref.rows
    assert np.array_equal(cand, ref.cand) and np.array_equal(eact, ref.eact) and np.array_equal(vact, ref.vact)


def test_oracle_graph_stat_accumulation_is_never_reset():
    """GraphStatCpu::compute (graph_stat_cpu.tpp:46-70) declares its
    label -> count accumulation outside the vertex loop, so a vertex counts
    towards "at least i label-b neighbours" with the neighbours of every
    earlier vertex of its thread's block.  Hand-worked case: vertices
    0 (label 0), 1 (label 1), 2 (label 0); entries 0->1, 0->2, 1->0, 2->0;
    template: one edge between labels 0 and 1.  With one thread vertex 2
    (no label-1 neighbour) inherits vertex 0's count; with three threads
    (one vertex per block) it does not."""
    off = np.array([0, 2, 3, 4], np.uint64)
    adj = np.array([1, 2, 0, 0], np.uint32)
    lab = np.array([0, 1, 0], np.uint64)
    p_off, p_adj, p_lab = [0, 1, 2], [1, 0], [0, 1]
    cand = np.array([1, 2, 1], np.uint64)
    eact = np.ones(4, np.uint8)
    labels, vt, et, al = oracle.graph_stat(off, adj, lab, p_off, p_adj, p_lab, cand, eact, threads=1)
    assert labels.tolist() == [0, 1] and vt.tolist() == [2, 1]
    assert et.tolist() == [[2, 1], [1, 0]]
    assert al[0, 1, 1] == 2 and al[1, 0, 1] == 1 and al[0, 0].sum() == 0 and al[1, 1].sum() == 0
    _, _, _, al3 = oracle.graph_stat(off, adj, lab, p_off, p_adj, p_lab, cand, eact, threads=3)
    assert al3[0, 1, 1] == 1 and al3[1, 0, 1] == 1


STAT_CASES = C.synthetic_cases(include_big=False)[:10]


@pytest.mark.gpu
@pytest.mark.parametrize("case", STAT_CASES, ids=lambda c: c["name"])
def test_gpu_graph_stat_equals_oracle(case):
    """The device statistics (k_stat_counts, k_stat_accum) against the
    oracle's block-by-block loop on the same states: after LCC0 and one LCC
    pass, and after the pruning pipeline, for 1, 3 and 17 blocks."""
    g, p = C.make_graph(case), C.make_pattern(case)
    off, adj, lab = g.host_csr()
    g.to_device(0)
    q = pm.Query(g, pattern=p)
    q.step()
    q.step()
    states = []
    for phase in ("first pass", "pruned"):
        if phase == "pruned":
            q.prune()
        cand, eact, _ = q.export()
        for threads in (1, 3, 17):
            try:
                ref = oracle.graph_stat(off, adj, lab, p.offsets, p.adj, p.labels, cand, eact, threads=threads)
            except oracle.StatMissing:
                with pytest.raises(pm.PmError) as e:
                    q.graph_stat(threads)
                assert e.value.code == pm.PM_E_STATISTICS
                continue
            got = q.graph_stat(threads)
            for a, b in zip(got, ref):
                assert np.array_equal(a, b), (phase, threads)
            states.append((phase, threads))
    q.close()
    assert states
