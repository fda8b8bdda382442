"""Serving and batching (pm_server_*, pm_batch_run).

The contract: a request's results are the same whether it runs alone
(pm_query_run) or in a mix of concurrent requests on the server — the step
rows (timing columns excluded), the exact match count and the final state
(role sets, CSR-entry and vertex flags), bit for bit, since all of it is
integer work.  Admission never lets the charged device bytes of the running
requests exceed the budget.
"""
from __future__ import annotations

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from tests import cases as C
from tests import pmtest

SYNTH = {c["name"]: c for c in pmtest.load_synthetic_golden()}
# Templates known to finish in well under a second on the scale-12 graph.
MIX = ["c1_scale10_cycle4", "triangle_rep_s9", "path4_rep_s9", "fixture3_s9", "k4_rep_s8", "two_cycles_s10",
       "scale12_tds", "cycle4_rep_s9"]


def _graph():
    return C.make_graph(SYNTH["scale12_tds"]).to_device(0)


def _alone(g, p):
    q = pm.Query(g, pattern=p)
    rows = [r.as_tuple() for r in q.run()]
    cand, eact, vact = q.export()
    count = q.match_count
    q.close()
    return rows, count, cand, eact, vact


def test_server_needs_a_device_graph():
    g = pm.Graph.rmat(6, 4, seed=1)  # host only
    cfg = pm.ServerConfig(2, 0)
    import ctypes

    h = ctypes.c_void_p()
    status = pm.lib.pm_server_create(g._h, ctypes.byref(cfg), ctypes.byref(h))
    if pm.device_count() == 0:
        assert status == pm.PM_E_NO_DEVICE
    else:
        assert status == pm.PM_SUCCESS
        pm.lib.pm_server_destroy(h)


def test_server_rejects_zero_slots():
    import ctypes

    g = pm.Graph.rmat(6, 4, seed=1)
    cfg = pm.ServerConfig(0, 0)
    h = ctypes.c_void_p()
    assert pm.lib.pm_server_create(g._h, ctypes.byref(cfg), ctypes.byref(h)) == pm.PM_E_INVALID_ARG


@pytest.mark.gpu
def test_mix_equals_alone():
    g = _graph()
    patterns = [C.make_pattern(SYNTH[n]) for n in MIX]
    expected = [_alone(g, p) for p in patterns]
    with pm.Server(g, slots=4) as srv:
        tickets = [srv.submit(p, export_state=True) for p in patterns[:4]]
        # The rest arrive while the first ones run (continuous admission).
        srv.wait(tickets[0])
        tickets += [srv.submit(p, export_state=True) for p in patterns[4:]]
        for name, t, exp in zip(MIX, tickets, expected):
            r = srv.wait(t)
            assert r.status == pm.PM_SUCCESS, name
            rows = [x.as_tuple() for x in srv.records(t)]
            assert rows == exp[0], name
            assert r.match_count == exp[1], name
            cand, eact, vact = srv.export(t)
            assert np.array_equal(cand, exp[2]), name
            assert np.array_equal(eact, exp[3]), name
            assert np.array_equal(vact, exp[4]), name
            assert r.latency_ms >= r.run_ms >= 0 and r.queue_ms >= 0
            srv.release(t)
        st = srv.stats()
        assert st.done == len(MIX) and st.running == 0 and st.queued == 0
        assert st.bytes_in_use == 0


@pytest.mark.gpu
def test_admission_by_memory_budget():
    g = _graph()
    patterns = [C.make_pattern(SYNTH[n]) for n in MIX[:5]]
    expected = [_alone(g, p)[1] for p in patterns]
    charges = []
    import ctypes

    for p in patterns:
        b = ctypes.c_uint64()
        pm._check(pm.lib.pm_query_estimate_bytes(g._h, p.n, ctypes.byref(b)))
        charges.append(b.value)
    # Room for the largest request plus a little: at most one at a time
    # whenever two would exceed it.
    budget = max(charges) + min(charges) // 2
    with pm.Server(g, slots=4, memory_budget=budget) as srv:
        tickets = [srv.submit(p) for p in patterns]
        counts = [srv.wait(t).match_count for t in tickets]
        st = srv.stats()
        assert st.peak_bytes <= budget
        assert st.memory_budget == budget
    assert counts == expected


@pytest.mark.gpu
def test_request_above_budget_is_refused():
    g = _graph()
    with pm.Server(g, slots=2, memory_budget=1 << 20) as srv:
        with pytest.raises(pm.PmError) as ei:
            srv.submit(C.make_pattern(SYNTH["triangle_rep_s9"]))
        assert ei.value.code == pm.PM_E_ADMISSION_DENIED


@pytest.mark.gpu
def test_requests_overlap_on_the_gpu():
    g = _graph()
    patterns = [C.make_pattern(SYNTH[n]) for n in MIX]
    with pm.Server(g, slots=4) as srv:
        tickets = [srv.submit(p) for p in patterns]
        results = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert all(r.status == pm.PM_SUCCESS for r in results)
    # More than one request was admitted at once at some point.
    assert st.peak_bytes > max(r.charged_bytes for r in results)


@pytest.mark.gpu
def test_batch_run_equals_alone():
    g = _graph()
    patterns = [C.make_pattern(SYNTH[n]) for n in MIX]
    expected = [_alone(g, p)[1] for p in patterns]
    counts, statuses = pm.batch_run(g, patterns, slots=3)
    assert list(statuses) == [pm.PM_SUCCESS] * len(patterns)
    assert [int(c) for c in counts] == expected


@pytest.mark.gpu
def test_shutdown_with_queued_requests():
    g = _graph()
    srv = pm.Server(g, slots=1)
    for n in MIX:
        srv.submit(C.make_pattern(SYNTH[n]))
    srv.close()  # queued requests are cancelled, the running one finishes
    # The graph is still usable afterwards.
    assert _alone(g, C.make_pattern(SYNTH["triangle_rep_s9"]))[1] == _alone(
        g, C.make_pattern(SYNTH["triangle_rep_s9"]))[1]


def test_autotune_rejects_empty_list():
    import ctypes

    g = pm.Graph.rmat(6, 4, seed=1)
    r = pm.TuneResult()
    assert pm.lib.pm_autotune(g._h, None, 0, 4, ctypes.byref(r)) == pm.PM_E_INVALID_ARG


@pytest.mark.gpu
def test_autotune_keeps_results():
    """The tuner's choices change speed only: counts before and after match."""
    g = _graph()
    patterns = [C.make_pattern(SYNTH[n]) for n in MIX[:4]]
    before = [_alone(g, p)[1] for p in patterns]
    chosen = pm.autotune(g, patterns, max_per_group=2)
    assert chosen["runs"] > 0
    assert chosen["probes_memo"] + chosen["probes_plain"] >= 1
    assert chosen["seg_entries"] in (512, 1024)
    assert chosen["enum_tail_swap"] in (0, 2, 4, 8)
    assert chosen["walk_tail_swap"] in (0, 2, 4, 8)
    after = [_alone(g, p)[1] for p in patterns]
    assert after == before
    # Leave the defaults for the tests that follow.
    pm.lib.pm_set_enum_table_entries(8192)
    pm.lib.pm_set_enum_presplit_by_kind(32, 8)
    pm.lib.pm_set_walk_presplit(64)
    pm.lib.pm_set_walk_table_entries(8192)
    pm.lib.pm_set_enum_tail_swap(4)
    pm.lib.pm_set_walk_tail_swap(4)
    pm.lib.pm_set_enum_count_memo(1)
    pm.lib.pm_set_walk_tail_state_memo(1)
    pm.lib.pm_set_pair_tail(1, 1)
    pm.lib.pm_set_enum_second_split(256)
    g.set_hub_plan(32, 1024)
