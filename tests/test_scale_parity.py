"""Parity on the large configurations.

- RMAT scale 22 (4,194,304 vertices, ~130M CSR entries), 16 Zipf(1.0)
  labels, the 6-vertex template of two 4-cycles sharing an edge with
  distinct labels 0..5: every pruning row, every role set and every CSR-entry
  flag against the oracle; the match count against the oracle's count over
  a seeded sample of sources (every 1024th vertex), compared per sample, not
  scaled.  With distinct labels no memo test can block a walk, so the
  reference's alreadyMatched shortcut cannot change an outcome and the
  oracle may run its constraint walks on every host core.
- RMAT scale 24, the served workload's graph and stream: the seeded 1 %
  sample (requests 0, 100, ..., 1900) pruned on the GPU; every request the
  GPU prunes within its budget and the oracle (LCC sweeps on every core,
  constraint walks in the canonical one-thread order) finishes within its
  deadline is compared row for row and state for state.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from pattenmatching_sharedmemory_gb300 import templates as T
from tests import pmtest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def test_c2_rmat22_two_cycles_full_state_and_sampled_count():
    from oracle import oracle

    g = pm.Graph.rmat(22, 16, 0.57, 0.19, 0.19, seed=1, permute=True).assign_labels("zipf", 16, 1.0, 1)
    p = T.two_cycles_sharing_edge([0, 1, 2, 3, 4, 5])
    off, adj, lab = g.host_csr()
    ref = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, threads=THREADS, nlcc_threads=THREADS,
                        stop_before_enumeration=True, deadline_ms=600000)
    g.to_device(0)
    q = pm.Query(g, pattern=p)
    rows = [r.as_tuple() for r in q.prune()]
    assert rows == ref.rows
    assert any(r[0] == "CC" for r in rows)
    cand, eact, vact = q.export()
    assert np.array_equal(cand, ref.cand)
    assert np.array_equal(eact, ref.eact)
    assert np.array_equal(vact, ref.vact)
    # Sampled count: the oracle's ENUMERATION over sources v % 1024 == 0
    # against the GPU walker over the same sources (integer counts: exact).
    stride = 1024
    role = oracle.enumeration_start_role(p.offsets, p.adj, p.labels)
    ref_s = oracle.run_ex(off, adj, lab, p.offsets, p.adj, p.labels, threads=THREADS, nlcc_threads=THREADS,
                          enum_sample_stride=stride, deadline_ms=600000, want_state=False)
    want = ref_s.match_count
    got = pmtest.sampled_count_gpu(g, p, cand, eact, role, stride)
    assert got == want
    assert want > 0
    # The whole count on the GPU is at least the sampled part.
    full = [r.as_tuple() for r in q.run()]
    assert full[-2][0] == "ENUMERATION" and full[-2][8] >= want
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
                                    stop_before_enumeration=True, deadline_ms=20000)
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
