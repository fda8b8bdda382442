#!/usr/bin/env python3
"""Benchmark of the GB300 PruneJuice pipeline (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c1|c2]

Workload c1 (default): undirected RMAT scale 16 (65,536 vertices, edge factor
16, a/b/c = .57/.19/.19, seed 1, self-loops and duplicates removed), labels
uniform over 5 values (seed 1); template: 4-cycle with labels 0,1,2,3.  A
step is one query through the full reference pipeline — LCC0, LCC to a
fixpoint, the CC constraint, LCC, exact ENUMERATION — on the resident graph.
Workload c2: RMAT scale 22, 16 Zipf(1.0) labels, the 6-vertex two-cycle
template on labels 10..15 (on frequent labels the exact count of that template
has over 1e10 embeddings and does not finish within minutes).

value  : queries/s with the graph resident in HBM (CUDA events around the
         timed steps, synchronize on both sides).
e2e    : queries/s through the C ABI from host buffers: every step uploads
         the CSR from pinned host memory (pm_graph_from_csr), creates the
         query, runs it and reads the role sets back (pm_query_export).
roofline: the dominant kernel class of the step (by device time), its
         algorithmic bytes over its CUDA-event time, against the measured
         HBM copy bandwidth.  Walker bytes: 16 B of CSR offsets per hop plus,
         per tested CSR entry, 4 B neighbour id + 1/8 B edge bit + 1/8 B
         active bit + ceil(k/8) B neighbour roles.
cpu_baseline: the oracle restatement of the reference (all host cores) on a
         bounded sample: CC/ENUMERATION sources sampled 1 in --sample-stride,
         their time scaled back up.
--impl reference: that CPU estimate as the reference arm.
Multi-GPU: replicas only — every rank runs its own queries on its own
graph replica; value = all ranks' queries / slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "c1": {"name": "rmat16_cycle4_full_pipeline", "scale": 16, "ef": 16, "labels": ("uniform", 5, 1.0, 1),
           "template": ("cycle", [0, 1, 2, 3]), "sample_stride": 32},
    "c2": {"name": "rmat22_two_cycles_rare_labels_full_pipeline", "scale": 22, "ef": 16,
           "labels": ("zipf", 16, 1.0, 1), "template": ("two_cycles", [10, 11, 12, 13, 14, 15]),
           "sample_stride": 1024},
}


def make_inputs(w):
    import pattenmatching_sharedmemory_gb300 as pm
    from pattenmatching_sharedmemory_gb300 import templates as T

    kind, n, s, seed = w["labels"]
    g = pm.Graph.rmat(w["scale"], w["ef"], 0.57, 0.19, 0.19, seed=1, permute=True).assign_labels(kind, n, s, seed)
    tk, labels = w["template"]
    tmpl = T.cycle(labels) if tk == "cycle" else T.two_cycles_sharing_edge(labels)
    return g, tmpl


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel: str):
    """dram bytes per launch recorded from an ncu capture (profiles/*.md)."""
    for f in (ROOT / "profiles").glob("*.md"):
        for line in f.read_text().splitlines():
            if line.startswith(f"traffic_bytes_per_launch[{kernel}]:"):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def kernel_class(step_name: str) -> str:
    return {"LCC0": "lcc", "LCC": "lcc", "CC": "walk", "PC": "walk", "TDS": "walk", "ENUMERATION": "enumerate"}.get(
        step_name, "other")


def run_gb300(args, w, rank, world):
    import torch

    import pattenmatching_sharedmemory_gb300 as pm

    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    g, tmpl = make_inputs(w)
    g.to_device(device)
    k_word = 1 if tmpl.n <= 8 else 4 if tmpl.n <= 24 else 8 if tmpl.n <= 56 else 16

    def one_query():
        q = pm.Query(g, pattern=tmpl)
        recs = q.run()
        return q, recs

    for _ in range(args.warmup):
        q, recs = one_query()
        q.close()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = int(pm.lib.pm_kernel_launches())
    per_class_ms = {}
    per_class_bytes = {}
    match = None
    lat = []
    # The c1 inputs (7.3 MB CSR) fit in the 129 MB L2: every timed step is
    # preceded, outside its timed interval, by a 512 MB write that flushes L2.
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{device}")
    elapsed_ms = 0.0
    with ClockSampler(device) as clocks:
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            start.record()
            t0 = time.perf_counter()
            q, recs = one_query()
            torch.cuda.synchronize()
            end.record()
            end.synchronize()
            lat.append((time.perf_counter() - t0) * 1e3)
            elapsed_ms += start.elapsed_time(end)
            match = q.match_count
            for i, r in enumerate(recs[:-1]):
                name = pm.STEP_NAMES[r.step]
                c = kernel_class(name)
                per_class_ms[c] = per_class_ms.get(c, 0.0) + r.step_ms
                scanned, hops = q.step_walk_stats(i)
                if c in ("walk", "enumerate"):
                    # NLCC hop formula: per hop 16 B of offsets, per tested
                    # entry 4 B id + 1/8 B edge bit + 1/8 B active bit +
                    # ceil(k/8) B neighbour roles.
                    b = hops * 16 + scanned * (4 + 0.25 + k_word)
                    per_class_bytes[c] = per_class_bytes.get(c, 0.0) + b
            q.close()
    del flush
    launches = int(pm.lib.pm_kernel_launches()) - launches0
    t = torch.tensor([elapsed_ms], device=f"cuda:{device}")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    elapsed_max = float(t.item())

    # e2e: host buffers through the C ABI
    off, adj, lab = g.host_csr()
    pin_off = torch.from_numpy(off.copy()).pin_memory()
    pin_adj = torch.from_numpy(adj.copy()).pin_memory()
    pin_lab = torch.from_numpy(lab.copy()).pin_memory()
    h2d = pin_off.numel() * 8 + pin_adj.numel() * 4 + pin_lab.numel() * 8
    d2h = g.vertex_count * (8 + 1) + g.edge_count
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        ge = pm.Graph.from_csr(pin_off.numpy(), pin_adj.numpy(), pin_lab.numpy(), device=device)
        qe = pm.Query(ge, pattern=tmpl)
        qe.run()
        cand, eact, vact = qe.export()
        qe.close()
        ge.close()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_t = torch.tensor([e2e_s], device=f"cuda:{device}")
    if world > 1:
        torch.distributed.all_reduce(e2e_t, op=torch.distributed.ReduceOp.MAX)
    e2e_qps = world * max(1, args.steps) / float(e2e_t.item())

    dom = max(per_class_ms, key=per_class_ms.get)
    peak, peak_kind = measured_peaks()
    n_launch_dom = sum(1 for r in recs[:-1] if kernel_class(pm.STEP_NAMES[r.step]) == dom) * args.steps
    achieved = None
    if dom in per_class_bytes and per_class_ms[dom] > 0:
        achieved = per_class_bytes[dom] / (per_class_ms[dom] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "peak_source": peak_kind,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                "traffic": profile_traffic(dom), "launches_in_timed_region": n_launch_dom,
                "kernel_ms_per_step": per_class_ms[dom] / args.steps,
                "note": "latency-bound depth-first walk; bytes are the per-hop algorithmic bytes"}
    qps = world * args.steps / (elapsed_max / 1e3)
    lat.sort()
    out = {
        "metric": "queries/s (full PruneJuice pipeline per query: LCC0, LCC fixpoint, NLCC, exact ENUMERATION)",
        "value": qps, "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": elapsed_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32/u64 integer and bitwise", "data": "synthetic (seeded RMAT + labels; reference datasets absent)",
        "config": {"workload": w["name"], "graph": f"rmat scale {w['scale']} ef {w['ef']}",
                   "vertices": g.vertex_count, "csr_entries": g.edge_count, "labels": list(w["labels"]),
                   "template": list(w["template"]), "match_count": match, "parallelism": f"replicas x{world}",
                   "l2": "flushed before every timed step (512 MB write outside the timed interval)",
                   "latency_ms_p50": lat[len(lat) // 2], "latency_ms_p99": lat[min(len(lat) - 1, int(len(lat) * 0.99))]},
        "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "per_class_ms_per_step": {k: v / args.steps for k, v in per_class_ms.items()},
        "clocks": clocks.summary(),
        "gpu_launches": launches,
    }
    return out, g, tmpl


def cpu_estimate(w, g, tmpl, stride, threads):
    """Oracle timing sample: LCC-type steps in full, CC/PC/TDS/ENUMERATION
    sources sampled 1/stride and scaled up.  Returns (seconds per query, info)."""
    from oracle import oracle

    off, adj, lab = g.host_csr()
    t0 = time.perf_counter()
    r = oracle.run(off, adj, lab, tmpl.offsets, tmpl.adj, tmpl.labels, threads=threads, sample_stride=stride)
    wall = time.perf_counter() - t0
    est_ms = 0.0
    for row, ms in zip(r.rows, r.timings):
        est_ms += ms * (stride if row[0] in ("CC", "PC", "TDS", "ENUMERATION") else 1)
    return est_ms / 1e3, {"sample_wall_s": wall, "stride": stride}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c1", choices=sorted(WORKLOADS))
    ap.add_argument("--sample-stride", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    stride = args.sample_stride or w["sample_stride"]
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        import pattenmatching_sharedmemory_gb300 as pm  # host-only graph generation

        g, tmpl = make_inputs(w)
        # Size the sample so the whole K + W run stays within ~3 minutes.
        _, probe = cpu_estimate(w, g, tmpl, stride, threads)
        target = max(1.0, 150.0 / max(1, args.steps + args.warmup))
        if probe["sample_wall_s"] > target:
            stride = int(stride * (probe["sample_wall_s"] / target + 1))
        times = []
        for _ in range(args.warmup):
            cpu_estimate(w, g, tmpl, stride, threads)
        info = {}
        for _ in range(args.steps):
            s, info = cpu_estimate(w, g, tmpl, stride, threads)
            times.append(s)
        per_query = statistics.mean(times)
        v = 1.0 / per_query
        out = {"impl": "reference", "metric": "queries/s (full PruneJuice pipeline per query: LCC0, LCC fixpoint, "
               "NLCC, exact ENUMERATION)", "value": v, "unit": "queries/s", "n_gpus": args.gpus,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_query * 1e3, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "u32/u64 integer and bitwise",
               "data": "synthetic (seeded RMAT + labels)",
               "config": {"workload": w["name"], "graph": f"rmat scale {w['scale']} ef {w['ef']}",
                          "template": list(w["template"])},
               "cpu_baseline": {"value": v, "unit": "queries/s", "cores": threads, "kind": "port",
                                "sample": f"oracle restatement, {threads} threads; CC/PC/TDS/ENUMERATION sources "
                                          f"sampled 1/{stride} and scaled x{stride}, LCC steps in full; "
                                          f"{info.get('sample_wall_s', 0):.1f} s per sample"},
               "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    out, g, tmpl = run_gb300(args, w, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            s, info = cpu_estimate(w, g, tmpl, stride, threads)
            out["cpu_baseline"] = {"value": 1.0 / s, "unit": "queries/s", "cores": threads, "kind": "port",
                                   "sample": f"oracle restatement, {threads} threads; CC/PC/TDS/ENUMERATION sources "
                                             f"sampled 1/{stride} and scaled x{stride}, LCC steps in full; "
                                             f"sample took {info['sample_wall_s']:.1f} s"}
        print(json.dumps(out))
    if world > 1:
        import torch

        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
