#!/usr/bin/env python3
"""Benchmark of the GB300 PruneJuice pipeline (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--slots S] [--lcc-scale L]

Graph: undirected RMAT scale 16 (65,536 vertices, edge factor 16, a/b/c =
.57/.19/.19, seed 1, self-loops and duplicates removed), labels uniform over
5 values (seed 1), resident on the GPU.  Stream: the 15 4-cycle templates
with four distinct labels (every choice of 4 of the 5 labels in its 3 cyclic
orders; labels 0,1,2,3 in that order is the classic single-query case).
Every request runs the full reference pipeline: LCC0, LCC to a fixpoint, the
CC constraint, LCC, exact ENUMERATION.

A step serves the whole stream: all 15 requests are submitted at once to a
server with S slots (continuous batching, admission by device memory) and
the step ends when the last one finished.  Before timing, pm_autotune picks
the LCC degree classes and the enumeration slicing / count-memo size on
probes of the stream (config.autotuned).

value      : served queries/s (host clock around the step, device
             synchronised on both sides; the requests run on S streams).
one_at_a_time: the same 15 templates run back to back through pm_query_run,
             queries/s and latency p50/p99, measured in the same process.
e2e        : served queries/s through the C ABI from host buffers: every
             step uploads the CSR from pinned host memory (pm_graph_from_csr),
             serves the stream and reads back every request's final state
             (role sets, CSR-entry and vertex flags) and rows.
roofline   : the dominant kernel class of a query run alone (by device
             time): its algorithmic bytes over its CUDA-event time against
             the measured HBM copy bandwidth.  Walker bytes: 16 B of CSR
             offsets per hop plus, per tested CSR entry, 4 B neighbour id +
             1/8 B edge bit + 1/8 B active bit + ceil(k/8) B neighbour roles.
small_stream: served vs one-at-a-time on 35 small requests (the triangles
             over the 5 labels, repeats allowed) on the same graph.
lcc_roofline: LCC passes on RMAT scale L (default 22; 16 Zipf labels, the
             two-cycle template on labels 0..5): per pass 1/8 B of edge bits
             per listed CSR entry plus, per gathered entry, 4 B neighbour id
             and the neighbour's packed word.
cpu_baseline: the oracle restatement of the reference (all host cores) on a
             bounded sample: each template's CC/ENUMERATION sources sampled
             1 in --sample-stride and the time scaled back up.
--impl reference: that CPU estimate of the same stream as the reference arm.
Multi-GPU: replicas only; every rank serves the stream on its own graph
replica; value = all ranks' queries / slowest rank's time.
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

WORKLOAD = {"name": "rmat16_cycle4_stream15_served", "scale": 16, "ef": 16, "labels": ("uniform", 5, 1.0, 1),
            "sample_stride": 256, "reference_stride": 512}


def stream_templates():
    """The 15 distinct-label 4-cycles over labels 0..4."""
    import itertools

    from pattenmatching_sharedmemory_gb300 import templates as T

    out = []
    for a, b, c, d in itertools.combinations(range(5), 4):
        for order in ([a, b, c, d], [a, b, d, c], [a, c, b, d]):
            out.append(T.cycle(order))
    return out


def small_templates():
    """The 35 triangles over labels 0..4 (labels may repeat)."""
    import itertools

    from pattenmatching_sharedmemory_gb300 import templates as T

    return [T.cycle(list(c)) for c in itertools.combinations_with_replacement(range(5), 3)]


def make_graph(w):
    import pattenmatching_sharedmemory_gb300 as pm

    kind, n, s, seed = w["labels"]
    return pm.Graph.rmat(w["scale"], w["ef"], 0.57, 0.19, 0.19, seed=1, permute=True).assign_labels(kind, n, s, seed)


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


def max_over_ranks(x: float, world: int, device: str) -> float:
    """Slowest rank's value (torch.distributed MAX all-reduce; `device` is the
    tensor device of the process group's backend)."""
    if world <= 1:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, world: int, slowest_seconds: float) -> float:
    """Whole-job throughput of `world` independent replicas: every rank's
    units over the slowest rank's time."""
    return world * units_per_rank / slowest_seconds


def word_bytes(k: int) -> int:
    return 2 if k <= 8 else 4 if k <= 24 else 8 if k <= 56 else 16


def pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(round(q * (len(xs) - 1))))]


def lcc_pass_bytes(listed: int, edges_eliminated: int, k: int) -> float:
    """Algorithmic bytes of one LCC pass, per entry of every checked list:
    neighbour id 4 B, its edge bit and active bit 1/8 B each, its label 1 B
    and its ceil(k/8) B of roles; plus 1/8 B written per eliminated entry.
    The per-vertex terms (offsets, own label and roles) are left out, so this
    is a lower bound."""
    return listed * (4 + 0.125 + 0.125 + 1 + (k + 7) // 8) + edges_eliminated / 8


def lcc_roofline(scale: int, device: int):
    """LCC passes on a CSR larger than L2: algorithmic bytes / step time."""
    import pattenmatching_sharedmemory_gb300 as pm
    from pattenmatching_sharedmemory_gb300 import templates as T

    g = pm.Graph.rmat(scale, 16, 0.57, 0.19, 0.19, seed=1, permute=True).assign_labels("zipf", 16, 1.0, 1)
    g.to_device(device)
    q = pm.Query(g, pattern=T.two_cycles_sharing_edge([0, 1, 2, 3, 4, 5]))
    wb = word_bytes(6)
    passes = []
    row = 0
    while True:
        rec, fin = q.step()
        name = pm.STEP_NAMES[rec.step]
        listed, gathered = q.step_walk_stats(row)
        row += 1
        if name == "LCC":
            passes.append((rec.step_ms, lcc_pass_bytes(listed, rec.results.edge_eliminated, 6), listed, gathered,
                           listed / 8 + gathered * (4 + wb)))
            if rec.results.vertex_eliminated == 0 and rec.results.edge_eliminated == 0:
                break
        if fin or row > 40:
            break
    q.close()
    peak, peak_kind = measured_peaks()
    ms = sum(p[0] for p in passes)
    by = sum(p[1] for p in passes)
    touched = sum(p[4] for p in passes)
    achieved = by / (ms / 1e3) / 1e9 if ms else None
    out = {"bound": "hbm", "kernel": "lcc sweep (k_lcc_check x2 + sweep 2)", "graph": f"rmat scale {scale} ef 16",
           "csr_entries": g.edge_count, "passes": len(passes), "ms_per_pass": ms / max(1, len(passes)),
           "pass_ms": [round(p[0], 3) for p in passes], "listed_per_pass": [p[2] for p in passes],
           "gathered_per_pass": [p[3] for p in passes],
           "bytes": "per checked-list entry 4 + 1/8 + 1/8 + 1 + ceil(k/8) B, + 1/8 B per eliminated entry",
           "achieved": achieved, "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
           "frac": achieved / peak if achieved else None,
           "achieved_touched": touched / (ms / 1e3) / 1e9 if ms else None,
           "touched_bytes": "1/8 B per listed entry (live-target bit) + (4 + W) B per gathered entry",
           "traffic": profile_traffic("lcc")}
    g.close()
    return out


def poisson_stream(g, pm, tmpls, rate_qps: float, duration_s: float, slots: int, seed: int):
    """Requests drawn from `tmpls` arriving as a Poisson process at
    `rate_qps` for `duration_s` into one server; every arrival is admitted as
    slots and memory free up.  Reports the completed rate and the per-request
    latency (submit to result) percentiles."""
    import random

    rng = random.Random(seed)
    with pm.Server(g, slots=slots) as srv:
        for t in tmpls[:slots]:  # warm the slots (streams, captured loops)
            tk = srv.submit(t)
            srv.wait(tk)
            srv.release(tk)
        tickets = []
        t0 = time.perf_counter()
        next_t = t0
        while True:
            now = time.perf_counter()
            if now - t0 >= duration_s:
                break
            if now < next_t:
                time.sleep(min(next_t - now, 0.001))
                continue
            tickets.append(srv.submit(tmpls[rng.randrange(len(tmpls))]))
            next_t += rng.expovariate(rate_qps)
        results = [srv.wait(t) for t in tickets]
        t1 = time.perf_counter()
        for t in tickets:
            srv.release(t)
    lat = [r.latency_ms for r in results]
    bad = sum(1 for r in results if r.status != pm.PM_SUCCESS)
    return {"offered_qps": rate_qps, "requests": len(tickets), "failed": bad,
            "completed_qps": len(tickets) / (t1 - t0) if t1 > t0 else None,
            "latency_ms_p50": pct(lat, 0.5) if lat else None, "latency_ms_p99": pct(lat, 0.99) if lat else None}


def small_stream(g, args, pm, torch):
    """Served vs one-at-a-time on a stream of small requests (35 triangles)."""
    tm = small_templates()
    reps = max(1, args.steps)
    served_lat, seq_lat = [], []
    counts = None
    # One long-lived server, warmed up once, serves every timed burst.
    with pm.Server(g, slots=args.slots) as srv:
        for _ in range(max(1, args.warmup)):
            [srv.wait(srv.submit(t)) for t in tm]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            rs = [srv.wait(x) for x in [srv.submit(t) for t in tm]]
            served_lat += [r.latency_ms for r in rs]
            counts = [int(r.match_count) for r in rs]
        torch.cuda.synchronize()
        served = len(tm) * reps / (time.perf_counter() - t0)
    t0 = time.perf_counter()
    for _ in range(reps):
        seq_counts = []
        for t in tm:
            t1 = time.perf_counter()
            q = pm.Query(g, pattern=t)
            q.run()
            seq_counts.append(q.match_count)
            q.close()
            seq_lat.append((time.perf_counter() - t1) * 1e3)
    torch.cuda.synchronize()
    seq = len(tm) * reps / (time.perf_counter() - t0)
    if seq_counts != counts:
        raise RuntimeError("small stream: served and one-at-a-time counts differ")
    return {"templates": "35 triangles over labels 0..4 (repeats allowed)", "requests_per_step": len(tm),
            "served": served, "one_at_a_time": seq, "unit": "queries/s", "speedup": served / seq,
            "latency_ms_p50": pct(served_lat, 0.5), "latency_ms_p99": pct(served_lat, 0.99),
            "one_at_a_time_latency_ms_p50": pct(seq_lat, 0.5), "one_at_a_time_latency_ms_p99": pct(seq_lat, 0.99)}


def run_gb300(args, w, rank, world):
    import torch

    import pattenmatching_sharedmemory_gb300 as pm

    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    pm._check(pm.lib.pm_set_lcc_graph(args.lcc_graph))
    g = make_graph(w)
    g.to_device(device)
    tmpls = stream_templates()
    n = len(tmpls)
    # Autotuner (outside the timed region): degree classes and enumeration
    # settings timed on probes of both streams, fastest kept in force.
    t_tune = time.perf_counter()
    tuned = pm.autotune(g, tmpls + small_templates(), max_per_group=4)
    tuned["seconds"] = round(time.perf_counter() - t_tune, 2)
    k_word = 1  # ceil(k/8) B of neighbour roles for the 4-vertex templates

    def serve_burst(srv, export=False):
        tickets = [srv.submit(t, export_state=export) for t in tmpls]
        results = [srv.wait(t) for t in tickets]
        states = [srv.export(t) for t in tickets] if export else None
        rows = [srv.records(t) for t in tickets] if export else None
        for t in tickets:
            srv.release(t)
        bad = [r.status for r in results if r.status != pm.PM_SUCCESS]
        if bad:
            raise RuntimeError(f"served requests failed: {bad}")
        return results, states, rows

    def serve_stream(graph, export=False):
        with pm.Server(graph, slots=args.slots) as srv:
            return serve_burst(srv, export)

    # The served measurement uses one long-lived server (created and warmed
    # up outside the timed region), as a serving process would.
    server = pm.Server(g, slots=args.slots)
    for _ in range(args.warmup):
        serve_burst(server)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = int(pm.lib.pm_kernel_launches())
    # The CSR (7.3 MB) fits in the 129 MB L2: every timed step is preceded,
    # outside its timed interval, by a 512 MB write that flushes L2.
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{device}")
    served_s = 0.0
    served_lat = []
    counts = None
    with ClockSampler(device) as clocks:
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            results, _, _ = serve_burst(server)
            torch.cuda.synchronize()
            served_s += time.perf_counter() - t0
            served_lat += [r.latency_ms for r in results]
            counts = [int(r.match_count) for r in results]
    launches = int(pm.lib.pm_kernel_launches()) - launches0
    server.close()
    served_max = max_over_ranks(served_s, world, f"cuda:{device}")

    # One at a time: the same stream through pm_query_run, back to back.
    seq_s = 0.0
    seq_lat = []
    per_class_ms, per_class_bytes, per_class_launch = {}, {}, {}
    seq_counts = []
    for _ in range(max(1, args.steps // 2)):
        flush.fill_(1)
        torch.cuda.synchronize()
        seq_counts = []
        t0 = time.perf_counter()
        for tm in tmpls:
            t1 = time.perf_counter()
            q = pm.Query(g, pattern=tm)
            recs = q.run()
            seq_lat.append((time.perf_counter() - t1) * 1e3)
            seq_counts.append(q.match_count)
            for i, r in enumerate(recs[:-1]):
                c = kernel_class(pm.STEP_NAMES[r.step])
                per_class_ms[c] = per_class_ms.get(c, 0.0) + r.step_ms
                per_class_launch[c] = per_class_launch.get(c, 0) + 1
                scanned, hops = q.step_walk_stats(i)
                if c in ("walk", "enumerate"):
                    b = hops * 16 + scanned * (4 + 0.25 + k_word)
                    per_class_bytes[c] = per_class_bytes.get(c, 0.0) + b
            q.close()
        torch.cuda.synchronize()
        seq_s += time.perf_counter() - t0
    seq_steps = max(1, args.steps // 2)
    del flush
    if seq_counts != counts:
        raise RuntimeError("served and one-at-a-time match counts differ")

    # e2e: host buffers through the C ABI, results read back.
    off, adj, lab = g.host_csr()
    pin_off = torch.from_numpy(off.copy()).pin_memory()
    pin_adj = torch.from_numpy(adj.copy()).pin_memory()
    pin_lab = torch.from_numpy(lab.copy()).pin_memory()
    h2d = pin_off.numel() * 8 + pin_adj.numel() * 4 + pin_lab.numel() * 8 + sum(
        t.offsets.nbytes + t.adj.nbytes + t.labels.nbytes for t in tmpls)
    d2h = n * (g.vertex_count * (8 + 1) + g.edge_count)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        ge = pm.Graph.from_csr(pin_off.numpy(), pin_adj.numpy(), pin_lab.numpy(), device=device)
        _, states, rows = serve_stream(ge, export=True)
        d2h_rows = sum(len(r) for r in rows) * 80
        ge.close()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_qps = replica_throughput(n * max(1, args.steps), world, max_over_ranks(e2e_s, world, f"cuda:{device}"))

    dom = max(per_class_ms, key=per_class_ms.get)
    peak, peak_kind = measured_peaks()
    achieved = None
    if dom in per_class_bytes and per_class_ms[dom] > 0:
        achieved = per_class_bytes[dom] / (per_class_ms[dom] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "peak_source": peak_kind,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "traffic": profile_traffic(dom),
                "steps_timed": per_class_launch.get(dom, 0),
                "kernel_ms_per_query": per_class_ms[dom] / (n * seq_steps),
                "note": "one query alone; latency-bound depth-first walk; bytes are the per-hop algorithmic bytes"}
    qps = replica_throughput(n * args.steps, world, served_max)
    seq_qps = n * seq_steps / seq_s
    out = {
        "metric": "queries/s served (continuous batching) vs one-at-a-time, full PruneJuice pipeline per query",
        "value": qps, "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": served_max / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32/u64 integer and bitwise",
        "data": "synthetic (seeded RMAT + labels; reference datasets absent)",
        "config": {"workload": w["name"], "graph": f"rmat scale {w['scale']} ef {w['ef']}",
                   "vertices": g.vertex_count, "csr_entries": g.edge_count, "labels": list(w["labels"]),
                   "templates": "15 distinct-label 4-cycles over labels 0..4", "requests_per_step": n,
                   "slots": args.slots, "arrival": "all requests of a step submitted at once",
                   "server": "one long-lived server across the timed steps (e2e: one per step, new graph upload)",
                   "autotuned": tuned,
                   "lcc_fixpoint": ("one CUDA graph launch per fixpoint (conditional WHILE node over a pass)"
                                    if args.lcc_graph else "host-driven, one launch sequence per pass"),
                   "match_counts": counts, "parallelism": f"replicas x{world}",
                   "l2": "flushed before every timed step (512 MB write outside the timed interval)"},
        "latency_ms": {"p50": pct(served_lat, 0.5), "p99": pct(served_lat, 0.99)},
        "one_at_a_time": {"value": seq_qps, "unit": "queries/s", "latency_ms_p50": pct(seq_lat, 0.5),
                          "latency_ms_p99": pct(seq_lat, 0.99)},
        "speedup_vs_one_at_a_time": qps / world / seq_qps,
        "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h + d2h_rows},
        "roofline": roofline,
        "per_class_ms_per_query": {k: v / (n * seq_steps) for k, v in per_class_ms.items()},
        "clocks": clocks.summary(),
        "gpu_launches": launches,
    }
    out["small_stream"] = small_stream(g, args, pm, torch)
    # Poisson arrivals of the same 15 templates at 50 % and 90 % of the burst
    # capacity measured above (extra figures: a failure here is reported, the
    # main line stands).
    try:
        out["poisson"] = [poisson_stream(g, pm, tmpls, f * qps / world, 4.0, args.slots, seed=11 + i)
                          for i, f in enumerate((0.5, 0.9))]
    except Exception as e:  # noqa: BLE001
        out["poisson"] = {"error": f"{type(e).__name__}: {e}"}
    if args.lcc_scale:
        out["lcc_roofline"] = lcc_roofline(args.lcc_scale, device)
    return out, g, tmpls


def cpu_estimate(g, tmpls, stride, threads):
    """Oracle timing sample of the stream: per template, LCC-type steps in
    full, CC/PC/TDS/ENUMERATION sources sampled 1/stride and scaled up.
    Returns (seconds for the whole stream, info)."""
    from oracle import oracle

    off, adj, lab = g.host_csr()
    t0 = time.perf_counter()
    est_ms = 0.0
    for tm in tmpls:
        r = oracle.run(off, adj, lab, tm.offsets, tm.adj, tm.labels, threads=threads, sample_stride=stride)
        for row, ms in zip(r.rows, r.timings):
            est_ms += ms * (stride if row[0] in ("CC", "PC", "TDS", "ENUMERATION") else 1)
    return est_ms / 1e3, {"sample_wall_s": time.perf_counter() - t0, "stride": stride}


def cpu_line(v, threads, stride, info, n):
    return {"value": v, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"oracle restatement, {threads} threads, all {n} templates of the stream; "
                      f"CC/PC/TDS/ENUMERATION sources sampled 1/{stride} and scaled x{stride}, LCC steps in "
                      f"full; {info.get('sample_wall_s', 0):.1f} s per sampled stream"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--lcc-scale", type=int, default=22)
    ap.add_argument("--sample-stride", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lcc-graph", type=int, default=1, choices=[0, 1],
                    help="run each LCC fixpoint as one CUDA graph (1) or one host-driven launch sequence per pass (0)")
    args = ap.parse_args()
    w = WORKLOAD
    stride = args.sample_stride or w["sample_stride"]
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        g = make_graph(w)  # host-only graph generation
        tmpls = stream_templates()
        n = len(tmpls)
        stride = args.sample_stride or w["reference_stride"]
        # Size the sample so the whole K + W run stays within ~3 minutes.
        _, probe = cpu_estimate(g, tmpls, stride, threads)
        target = max(1.0, 150.0 / max(1, args.steps + args.warmup))
        if probe["sample_wall_s"] > target:
            stride = int(stride * (probe["sample_wall_s"] / target + 1))
        for _ in range(args.warmup):
            cpu_estimate(g, tmpls, stride, threads)
        times, info = [], {}
        for _ in range(args.steps):
            sec, info = cpu_estimate(g, tmpls, stride, threads)
            times.append(sec)
        per_stream = statistics.mean(times)
        v = n / per_stream
        out = {"impl": "reference",
               "metric": "queries/s served (continuous batching) vs one-at-a-time, full PruneJuice pipeline per query",
               "value": v, "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": per_stream * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "u32/u64 integer and bitwise", "data": "synthetic (seeded RMAT + labels)",
               "config": {"workload": w["name"], "graph": f"rmat scale {w['scale']} ef {w['ef']}",
                          "templates": "15 distinct-label 4-cycles over labels 0..4", "requests_per_step": n},
               "cpu_baseline": cpu_line(v, threads, stride, info, n),
               "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    out, g, tmpls = run_gb300(args, w, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            sec, info = cpu_estimate(g, tmpls, stride, threads)
            out["cpu_baseline"] = cpu_line(len(tmpls) / sec, threads, stride, info, len(tmpls))
        print(json.dumps(out))
    if world > 1:
        import torch

        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
