"""Failure handling, exercised without any GPU fault.

Every failure here is made on the host or by a bounded device-side wait:
- the walkers' step deadline (pm_set_walk_budget_ms) runs out on a case
  whose walks take longer, and the kernels return a timeout status;
- a request's wall-clock budget (pm_set_query_budget_ms) runs out;
- pm_server_wait gives up on a request that is still running;
- a queued or running request is cancelled (pm_server_cancel);
- a device allocation is made to fail by the host-side injector
  (pm_debug_fail_device_alloc_after), as an out-of-memory cudaMalloc would.
After each, the library must still work: the next query on the same graph
gives the golden rows, bit for bit (TOTEM's CHK convention of returning an
error code and carrying on, src/totem/totem_comdef.h:88-95).
"""
from __future__ import annotations

import pytest

import pattenmatching_sharedmemory_gb300 as pm
from tests import cases as C
from tests import pmtest

pytestmark = pytest.mark.gpu

SYNTH = {c["name"]: c for c in pmtest.load_synthetic_golden()}


@pytest.fixture(scope="module")
def c1():
    """The scale-16 4-cycle: ENUMERATION of 71.6M matches, ~15 ms of walks."""
    case = SYNTH["c1_scale16_cycle4"]
    g = C.make_graph(case).to_device(0)
    yield case, g, C.make_pattern(case)
    g.close()


def _rows(g, p):
    q = pm.Query(g, pattern=p)
    rows = [list(r.as_tuple()) for r in q.run()]
    q.close()
    return rows


def _expect_golden(case, g, p):
    assert _rows(g, p) == case["rows"]


def test_walk_budget_timeout_then_golden(c1):
    case, g, p = c1
    assert pm.lib.pm_set_walk_budget_ms(1.0) == pm.PM_SUCCESS
    try:
        q = pm.Query(g, pattern=p)
        with pytest.raises(pm.PmError) as e:
            q.run()
        assert e.value.code == pm.PM_E_TIMEOUT
        assert "budget" in str(e.value)
        # The step the deadline cut short: a walker step with no result
        # row, its device time and the entries its walkers tested.
        kind, ms, scanned, hops = q.aborted_step()
        assert pm.STEP_NAMES[kind] in ("CC", "ENUMERATION") and ms > 0 and scanned > 0
        q.close()
    finally:
        assert pm.lib.pm_set_walk_budget_ms(120000.0) == pm.PM_SUCCESS
    _expect_golden(case, g, p)
    q = pm.Query(g, pattern=p)
    q.run()
    assert q.aborted_step() is None
    q.close()


def test_query_budget_timeout_then_golden(c1):
    case, g, p = c1
    assert pm.lib.pm_set_query_budget_ms(2.0) == pm.PM_SUCCESS
    try:
        q = pm.Query(g, pattern=p)
        with pytest.raises(pm.PmError) as e:
            q.run()
        assert e.value.code == pm.PM_E_TIMEOUT
        q.close()
        # Served requests end the same way, and the slot stays usable.
        with pm.Server(g, slots=1) as srv:
            r = srv.wait(srv.submit(p))
            assert r.status == pm.PM_E_TIMEOUT
    finally:
        assert pm.lib.pm_set_query_budget_ms(0.0) == pm.PM_SUCCESS
    with pm.Server(g, slots=1) as srv:
        t = srv.submit(p)
        assert srv.wait(t).status == pm.PM_SUCCESS
        assert [list(r.as_tuple()) for r in srv.records(t)] == case["rows"]
    assert pm.lib.pm_set_query_budget_ms(-1.0) == pm.PM_E_INVALID_ARG


def test_server_wait_zero_timeout_on_running_request(c1):
    case, g, p = c1
    with pm.Server(g, slots=1) as srv:
        t = srv.submit(p)
        with pytest.raises(pm.PmError) as e:
            srv.wait(t, timeout_ms=0.0)
        assert e.value.code == pm.PM_E_TIMEOUT
        with pytest.raises(pm.PmError) as e:
            srv.release(t)  # still running: not releasable
        assert e.value.code == pm.PM_E_BUSY
        r = srv.wait(t)
        assert r.status == pm.PM_SUCCESS and r.match_count == case["rows"][-2][8]


def test_cancel_queued_and_running(c1):
    case, g, p = c1
    with pm.Server(g, slots=1) as srv:
        running = srv.submit(p)
        queued = [srv.submit(p) for _ in range(3)]
        srv.cancel(queued[1])
        r = srv.wait(queued[1])
        assert r.status == pm.PM_E_CANCELLED and r.run_ms == 0.0
        srv.cancel(running)
        assert srv.wait(running).status in (pm.PM_E_CANCELLED, pm.PM_SUCCESS)
        for t in (queued[0], queued[2]):
            r = srv.wait(t)
            assert r.status == pm.PM_SUCCESS
            assert [list(x.as_tuple()) for x in srv.records(t)] == case["rows"]
        srv.cancel(queued[0])  # finished: left as it is
        assert srv.wait(queued[0]).status == pm.PM_SUCCESS
        with pytest.raises(pm.PmError) as e:
            srv.cancel(10 ** 9)
        assert e.value.code == pm.PM_E_INVALID_ARG


def test_cancel_running_request_stops_between_steps():
    """A template with many constraint steps: cancelling it while it runs
    ends it before the schedule finishes."""
    case = SYNTH["scale12_tds"]
    g = C.make_graph(case).to_device(0)
    p = C.make_pattern(case)
    with pm.Server(g, slots=1) as srv:
        t = srv.submit(p)
        srv.cancel(t)
        r = srv.wait(t)
        assert r.status in (pm.PM_E_CANCELLED, pm.PM_SUCCESS)
        if r.status == pm.PM_E_CANCELLED:
            assert r.n_records < len(case["rows"])
        t2 = srv.submit(p)
        assert srv.wait(t2).status == pm.PM_SUCCESS
        assert [list(x.as_tuple()) for x in srv.records(t2)] == case["rows"]
    g.close()


def test_injected_device_oom_then_golden():
    """Fail the n-th device allocation of a whole query (creation and every
    step's buffers) for each n in turn: the call returns PM_E_OOM with no
    leak or poisoned state, until n passes the query's allocation count."""
    case = SYNTH["scale12_tds"]
    g = C.make_graph(case).to_device(0)
    p = C.make_pattern(case)
    failures = 0
    try:
        for n in range(0, 200):
            assert pm.lib.pm_debug_fail_device_alloc_after(n) == pm.PM_SUCCESS
            try:
                q = pm.Query(g, pattern=p)
                rows = [list(r.as_tuple()) for r in q.run()]
                q.close()
            except pm.PmError as e:
                assert e.code == pm.PM_E_OOM, e
                assert "injected" in str(e)
                failures += 1
                continue
            assert rows == case["rows"]
            break
        else:
            pytest.fail("the query made more than 200 device allocations")
    finally:
        pm.lib.pm_debug_fail_device_alloc_after(-1)
    assert failures >= 5
    # Served: the failing request reports PM_E_OOM, the slot carries on.
    with pm.Server(g, slots=1) as srv:
        pm.lib.pm_debug_fail_device_alloc_after(0)
        try:
            bad = srv.submit(p)
            assert srv.wait(bad).status == pm.PM_E_OOM
        finally:
            pm.lib.pm_debug_fail_device_alloc_after(-1)
        ok = srv.submit(p)
        assert srv.wait(ok).status == pm.PM_SUCCESS
        assert [list(x.as_tuple()) for x in srv.records(ok)] == case["rows"]
    assert _rows(g, p) == case["rows"]
    g.close()


def test_prune_only_matches_oracle_then_full_run():
    """pm_query_prune stops where the schedule would enter ENUMERATION; the
    rows equal the oracle's pruning-only run, and a following pm_query_run
    finishes with the golden rows."""
    from oracle import oracle

    for name in ("two_cycles_zipf_s10", "scale12_tds", "k4_rep_s8"):
        case = SYNTH[name]
        g = C.make_graph(case)
        p = C.make_pattern(case)
        off, adj, lab = g.host_csr()
        ref = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, stop_before_enumeration=True)
        g.to_device(0)
        q = pm.Query(g, pattern=p)
        rows = [r.as_tuple() for r in q.prune()]
        assert rows == ref.rows, name
        cand, eact, vact = q.export()
        assert (cand == ref.cand).all() and (eact == ref.eact).all() and (vact == ref.vact).all()
        full = [list(r.as_tuple()) for r in q.run()]
        assert full == case["rows"], name
        q.close()
        with pm.Server(g, slots=2) as srv:
            t = srv.submit(p, prune_only=True)
            r = srv.wait(t)
            assert r.status == pm.PM_SUCCESS and r.match_count == 0
            assert [x.as_tuple() for x in srv.records(t)] == ref.rows
        g.close()
