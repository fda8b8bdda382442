"""Parity on the large configurations.

- RMAT scale 22 (4,194,304 vertices, ~130M CSR entries), 16 Zipf(1.0)
  labels, the 6-vertex template of two 4-cycles sharing an edge with
  distinct labels 0..5 (the oracle's first CC step alone takes the host
  cores many minutes, so its walks are checked on a source sample):
  LCC0 and the LCC fixpoint, every row, role set and CSR-entry flag; the
  first CC step's decisions for the sources v % 1024 == 0.  With distinct
  labels no memo test can block a walk, so the reference's alreadyMatched
  shortcut cannot change an outcome and the oracle may run its walks on
  every host core.  The steps after the first CC (the second 4-cycle, the
  6-cycle around both, the template-driven search, ENUMERATION) are out of
  reach here: single sources reach hubs of 10^5 entries, the oracle's
  sampled first CC alone takes a minute of 16 cores per 1/1024 of the
  sources, and the GPU's later walker steps run past its step budget.
- RMAT scale 24, the served workload's graph and stream: the seeded 1 %
  sample (requests 0, 100, ..., 1900) pruned on the GPU, in order, until
  five are compared: every request the GPU prunes within its budget and the
  oracle (LCC sweeps on every core, constraint walks in the canonical
  one-thread order) finishes within its deadline is compared row for row
  and state for state.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from pattenmatching_sharedmemory_gb300 import templates as T

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def test_c2_rmat22_two_cycles_state_and_sampled_counts():
    from oracle import oracle

    g = pm.Graph.rmat(22, 16, 0.57, 0.19, 0.19, seed=1, permute=True).assign_labels("zipf", 16, 1.0, 1)
    p = T.two_cycles_sharing_edge([0, 1, 2, 3, 4, 5])
    off, adj, lab = g.host_csr()
    # 1. LCC0 and the first LCC fixpoint: every row and the whole state.  A
    #    first oracle run whose walks visit no source (sample stride 2^40)
    #    finds where the schedule reaches the first CC step; a second one
    #    stops there.
    sched = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, threads=THREADS, nlcc_threads=THREADS,
                          stop_before_enumeration=True, max_steps=64, sample_stride=1 << 40, deadline_ms=600000,
                          want_state=False)
    m = next(i for i, r in enumerate(sched.rows) if r[0] == "CC")
    ref = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, threads=THREADS, nlcc_threads=THREADS,
                        stop_before_enumeration=True, max_steps=m, deadline_ms=600000)
    assert ref.rows[-1][0] == "CC" and ref.rows[:-1] == sched.rows[:m]
    g.to_device(0)
    q = pm.Query(g, pattern=p)
    rows = [q.step()[0].as_tuple() for _ in range(m)]
    assert rows == ref.rows[:-1]
    cand, eact, vact = q.export()
    assert np.array_equal(cand, ref.cand) and np.array_equal(eact, ref.eact) and np.array_equal(vact, ref.vact)
    # 2. The first CC step (distinct labels: each (vertex, role) decision is
    #    independent of the other sources'): the oracle walks the sources
    #    v % 1024 == 0 only (about a minute on 16 cores); their role sets
    #    after the step must agree.
    rec, _ = q.step()
    assert pm.STEP_NAMES[rec.step] == "CC"
    cand2, _, vact2 = q.export()
    ref2 = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, threads=THREADS, nlcc_threads=THREADS,
                         stop_before_enumeration=True, max_steps=m + 1, sample_stride=1024, deadline_ms=600000)
    assert ref2.rows[m][0] == "CC" and ref2.rows[m][7] > 0
    sampled = np.arange(g.vertex_count) % 1024 == 0
    assert np.array_equal(cand2[sampled], ref2.cand[sampled])
    assert np.array_equal(vact2[sampled], ref2.vact[sampled])
    assert (cand2[sampled] != cand[sampled]).any() or rec.results.match_eliminated == 0
    q.close()
    g.close()


def test_c4_rmat24_one_percent_sample():
    from oracle import oracle

    g = pm.Graph.rmat(24, 16, 0.57, 0.19, 0.19, seed=1, permute=True).assign_labels("zipf", 32, 1.2, 1)
    g.to_device(0)
    off, adj, lab = g.host_csr()
    stream = T.served_stream(2000)
    compared, gpu_timeouts, oracle_timeouts = [], 0, 0
    assert pm.lib.pm_set_query_budget_ms(3000.0) == pm.PM_SUCCESS
    try:
        for i in range(0, 2000, 100):
            if len(compared) >= 5:
                break
            p = stream[i]
            q = pm.Query(g, pattern=p)
            try:
                rows = [r.as_tuple() for r in q.prune()]
            except pm.PmError as e:
                assert e.code == pm.PM_E_TIMEOUT
                gpu_timeouts += 1
                q.close()
                continue
            cand, eact, vact = q.export()
            q.close()
            try:
                ref = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, threads=THREADS, nlcc_threads=1,
                                    stop_before_enumeration=True, deadline_ms=8000)
            except oracle.OracleTimeout:
                oracle_timeouts += 1
                continue
            assert rows == ref.rows, i
            assert np.array_equal(cand, ref.cand), i
            assert np.array_equal(eact, ref.eact), i
            assert np.array_equal(vact, ref.vact), i
            compared.append(i)
    finally:
        pm.lib.pm_set_query_budget_ms(0.0)
    print(f"compared {compared}, GPU timeouts {gpu_timeouts}, oracle timeouts {oracle_timeouts}")
    assert len(compared) >= 3
    g.close()
