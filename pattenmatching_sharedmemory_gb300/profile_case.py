"""Small, fixed cases for profiling single kernels (ncu) and for timing them.

    python -m pattenmatching_sharedmemory_gb300.profile_case c1 [--queries N]
        full pipeline of the bench workload (RMAT 16, 4-cycle), N queries
    python -m pattenmatching_sharedmemory_gb300.profile_case lcc22 [--scale S]
        LCC0 and the LCC fixpoint on RMAT scale S (default 22, 16 Zipf
        labels, two-cycle template on labels 0..5): the HBM-bound kernels
        k_lcc_check / k_apply on a CSR larger than L2; --hub-degree and
        --seg-entries set the LCC degree classes

Prints one line per step with its CUDA-event time, its eliminated vertices /
CSR entries and, for LCC, the CSR entries of the lists its sweep checked and
how many of them it read a neighbour word for.
"""
from __future__ import annotations

import argparse
import sys

import pattenmatching_sharedmemory_gb300 as pm
from pattenmatching_sharedmemory_gb300 import templates as T


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["c1", "lcc22"])
    ap.add_argument("--queries", type=int, default=1)
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--hub-degree", type=int, default=None, help="LCC hub threshold (CSR entries)")
    ap.add_argument("--seg-entries", type=int, default=2048, help="CSR entries per hub segment")
    a = ap.parse_args()
    if a.case == "c1":
        g = pm.Graph.rmat(16, 16, seed=1).assign_labels("uniform", 5, 1.0, 1).to_device(0)
        tmpl = T.cycle([0, 1, 2, 3])
        for _ in range(a.queries):
            q = pm.Query(g, pattern=tmpl)
            for r in q.run():
                print(pm.STEP_NAMES[r.step], f"{r.step_ms:.3f} ms", r.results.enumeration)
            q.close()
        return 0
    g = pm.Graph.rmat(a.scale, 16, seed=1).assign_labels("zipf", 16, 1.0, 1).to_device(0)
    if a.hub_degree is not None:
        g.set_hub_plan(a.hub_degree, a.seg_entries)
    q = pm.Query(g, pattern=T.two_cycles_sharing_edge([0, 1, 2, 3, 4, 5]))
    row = 0
    while True:
        rec, fin = q.step()
        name = pm.STEP_NAMES[rec.step]
        streamed, gathered = q.step_walk_stats(row)
        row += 1
        print(name, f"{rec.step_ms:.3f} ms", rec.results.vertex_eliminated, rec.results.edge_eliminated,
              f"listed={streamed} gathered={gathered} active_v={rec.active_vertex} active_e={rec.active_edge}")
        if name == "LCC" and rec.results.vertex_eliminated == 0 and rec.results.edge_eliminated == 0 and \
                rec.results.match_eliminated == 0:
            break
        if fin:
            break
    return 0


if __name__ == "__main__":
    sys.exit(main())
