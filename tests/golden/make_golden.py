"""Generates the golden fixtures under tests/golden/ from the reference itself.

Run in a container that has the reference sources and oracle/_ref built
(`make -C oracle ref`):

    python tests/golden/make_golden.py [--skip-c1]

It writes
  data/test_{1..4}/          the reference's bundled fixtures (inputs), copied
  expected_fixtures.json     the reference's rows / vertex / graph outputs on them
  synthetic_cases.json       seeded RMAT + template cases: generation
                             parameters and the reference's outputs (rows,
                             sha256 of vertex_NNNN / graph_NNNN, match count)
  constraints.json.gz        reference constraint dumps (log.totem) for
                             random templates
and, on request,
  --only stream15            stream15_rmat16.json: the RMAT-16 stream's 15
                             4-cycles (hours of CPU; entries appended as the
                             reference finishes them)
  --only article             article_variants.json (needs `make -C oracle
                             ref-article`)
  --only order               order_variants.json: the constraint-order
                             drivers (needs `make -C oracle ref-order`)
All reference runs use PM_REF_THREADS=1, the canonical sequential order,
unless an entry records another thread count.
"""
from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import pattenmatching_sharedmemory_gb300 as pm  # noqa: E402
from pattenmatching_sharedmemory_gb300 import templates as T  # noqa: E402
from tests import cases as C  # noqa: E402

# The reference checkout (read-only); PM_REFERENCE_DIR overrides the default.
REF_ROOT = Path(os.environ.get("PM_REFERENCE_DIR", "/root/reference"))
REF_DATA = REF_ROOT / "data" / "patternmatching"
REF_BIN = ROOT / "oracle" / "_ref" / "patternmatching"


def run_reference(graph, labels, pattern_dir, out_dir, threads=1, timeout=600, binary=None):
    out_dir = Path(out_dir)
    if out_dir.exists():
        shutil.rmtree(out_dir)
    bin_path = str(out_dir) + ".bin"
    if os.path.exists(bin_path):
        os.remove(bin_path)
    env = dict(os.environ, PM_REF_THREADS=str(threads))
    cmd = [str(binary or REF_BIN), "-i", str(graph), "-b", bin_path, "-v", str(labels), "-p", str(pattern_dir).rstrip("/") + "/",
           "-o", str(out_dir) + "/"]
    subprocess.run(cmd, env=env, check=True, timeout=timeout, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return parse_outputs(out_dir)


def parse_outputs(out_dir):
    out_dir = Path(out_dir)
    rows = []
    for line in (out_dir / "results.totem").read_text().splitlines()[1:]:
        f = [x.strip() for x in line.split(";")]
        rows.append([f[1]] + [int(x) for x in f[4:12]])
    last = int((out_dir / "results.totem").read_text().splitlines()[-1].split(";")[0])
    vtx = (out_dir / f"vertex_{last:04d}.totem").read_bytes()
    grp = (out_dir / f"graph_{last:04d}.totem").read_bytes()
    log = (out_dir / "log.totem").read_text()
    return {"rows": rows, "vertex": vtx, "graph": grp, "log": log, "last": last}


def constraint_section(log: str) -> str:
    """The constraint dump part of log.totem, timestamps and blank lines removed."""
    out, on = [], False
    for line in log.splitlines():
        if line.startswith("[") and "] : " in line:
            line = line.split("] : ", 1)[1]
        if line.startswith("Generate Local constraint"):
            on = True
        if line.startswith("Initialize LCC0"):
            break
        if on and line.strip():
            out.append(line.rstrip())
    return "\n".join(out)


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def fixtures():
    out = {}
    for t in ["test_1", "test_2", "test_3", "test_4"]:
        src = REF_DATA / t
        dst = HERE / "data" / t
        if dst.exists():
            shutil.rmtree(dst)
        shutil.copytree(src, dst)
        for p in dst.rglob("*"):
            os.chmod(p, 0o755 if p.is_dir() else 0o644)
        with tempfile.TemporaryDirectory() as tmp:
            res = run_reference(dst / "graph.totem", dst / "vertex_data" / "graph_vertex_data.totem",
                                dst / "pattern_1", Path(tmp) / "out")
        out[t] = {"rows": res["rows"], "vertex": res["vertex"].decode(), "graph": res["graph"].decode(),
                  "constraints": constraint_section(res["log"]), "last": res["last"]}
        print(t, res["rows"][-2])
    (HERE / "expected_fixtures.json").write_text(json.dumps(out, indent=1))


def synthetic(skip_big: bool, only_big: bool = False):
    results = []
    cases = C.synthetic_cases(include_big=not skip_big)
    if only_big:
        cases = [c for c in cases if c.get("big")]
    for case in cases:
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            g = C.make_graph(case)
            g.write_text(tmp / "g.totem", tmp / "labels.totem")
            p = C.make_pattern(case)
            p.write(tmp / "pattern")
            try:
                res = run_reference(tmp / "g.totem", tmp / "labels.totem", tmp / "pattern", tmp / "out",
                                    threads=case.get("ref_threads", 1), timeout=case.get("timeout", 300))
            except subprocess.TimeoutExpired:
                print("timeout", case["name"])
                continue
        entry = dict(case)
        entry.update({"rows": res["rows"], "vertex_sha256": sha(res["vertex"]), "graph_sha256": sha(res["graph"]),
                      "last": res["last"]})
        results.append(entry)
        print(case["name"], res["rows"][-2][8], "matches", len(res["rows"]), "rows")
    name = "synthetic_big.json" if only_big else "synthetic_cases.json"
    if not only_big:
        results = [r for r in results if not r.get("big")]
    (HERE / name).write_text(json.dumps(results, indent=1))


def stream15():
    """The RMAT-16 served stream's 15 4-cycles, one reference run each,
    appended to stream15_rmat16.json as they finish (hours of CPU)."""
    path = HERE / "stream15_rmat16.json"
    results = json.loads(path.read_text()) if path.exists() else []
    have = {r["name"] for r in results}
    for case in C.stream15_cases():
        if case["name"] in have:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            g = C.make_graph(case)
            g.write_text(tmp / "g.totem", tmp / "labels.totem")
            C.make_pattern(case).write(tmp / "pattern")
            res = run_reference(tmp / "g.totem", tmp / "labels.totem", tmp / "pattern", tmp / "out",
                                threads=case["ref_threads"], timeout=case["timeout"])
        entry = dict(case)
        entry.update({"rows": res["rows"], "vertex_sha256": sha(res["vertex"]), "graph_sha256": sha(res["graph"]),
                      "last": res["last"]})
        results.append(entry)
        path.write_text(json.dumps(results, indent=1))
        print(case["name"], res["rows"][-2][8], "matches", flush=True)


def article():
    """The article drivers' strict and backtrack variants
    (oracle/_ref/patternmatching_{strict,backtrack}, test_article/
    CMakeLists.txt:12-33) on the bundled fixtures and the small synthetic
    cases: rows and sha256 of the final vertex / graph files."""
    out = []
    cases = [("fixture_" + t, None, t) for t in ["test_1", "test_2", "test_3", "test_4"]]
    cases += [(c["name"], c, None) for c in C.synthetic_cases(include_big=False)
              if c["name"] not in ("scale12_cycle4",)]
    for name, case, fixture in cases:
        for variant in ("strict", "backtrack"):
            binary = ROOT / "oracle" / "_ref" / f"patternmatching_{variant}"
            with tempfile.TemporaryDirectory() as tmp:
                tmp = Path(tmp)
                if fixture:
                    d = HERE / "data" / fixture
                    graph, labels, pdir = d / "graph.totem", d / "vertex_data" / "graph_vertex_data.totem", \
                        d / "pattern_1"
                else:
                    g = C.make_graph(case)
                    g.write_text(tmp / "g.totem", tmp / "labels.totem")
                    C.make_pattern(case).write(tmp / "pattern")
                    graph, labels, pdir = tmp / "g.totem", tmp / "labels.totem", tmp / "pattern"
                try:
                    res = run_reference(graph, labels, pdir, tmp / "out", binary=binary, timeout=300)
                except subprocess.TimeoutExpired:
                    print("timeout", name, variant)
                    continue
            out.append({"name": name, "variant": variant, "fixture": fixture, "case": case, "rows": res["rows"],
                        "vertex_sha256": sha(res["vertex"]), "graph_sha256": sha(res["graph"]),
                        "last": res["last"]})
            print(name, variant, res["rows"][-1], flush=True)
    (HERE / "article_variants.json").write_text(json.dumps(out, indent=1))


ORDER_BINARIES = ("enumerate_intuitive", "effectiveness", "enumerate_effectiveness",
                  "enumerate_effectiveness_early")


def order():
    """The article's constraint-order drivers (oracle/_ref/
    patternmatching_order_*, test_article/CMakeLists.txt:53-73; backtrack
    walks with all three optimisations) on the bundled fixtures and the small
    synthetic cases, with one thread and, for a few cases, three (the graph
    statistics and the cost estimate depend on the thread count).  A run the
    reference ends by an uncaught exception (a graph statistic the estimate
    reads is absent) is recorded with "aborted": true.  An empty step name
    (the first row of the dynamic order) is recorded as "START"."""
    out = []
    cases = [("fixture_" + t, None, t) for t in ["test_1", "test_2", "test_3", "test_4"]]
    cases += [(c["name"], c, None) for c in C.synthetic_cases(include_big=False)
              if c["name"] not in ("scale12_cycle4",)]
    for ci, (name, case, fixture) in enumerate(cases):
        for binary_name in ORDER_BINARIES:
            for threads in ((1, 3) if ci % 4 == 1 else (1,)):
                binary = ROOT / "oracle" / "_ref" / f"patternmatching_order_{binary_name}"
                with tempfile.TemporaryDirectory() as tmp:
                    tmp = Path(tmp)
                    if fixture:
                        d = HERE / "data" / fixture
                        graph, labels, pdir = d / "graph.totem", d / "vertex_data" / "graph_vertex_data.totem", \
                            d / "pattern_1"
                    else:
                        g = C.make_graph(case)
                        g.write_text(tmp / "g.totem", tmp / "labels.totem")
                        C.make_pattern(case).write(tmp / "pattern")
                        graph, labels, pdir = tmp / "g.totem", tmp / "labels.totem", tmp / "pattern"
                    entry = {"name": name, "order": binary_name, "threads": threads, "fixture": fixture,
                             "case": case}
                    try:
                        res = run_reference(graph, labels, pdir, tmp / "out", binary=binary, timeout=300,
                                            threads=threads)
                    except subprocess.TimeoutExpired:
                        print("timeout", name, binary_name, flush=True)
                        continue
                    except subprocess.CalledProcessError as e:
                        entry.update({"aborted": True, "returncode": e.returncode})
                        out.append(entry)
                        print(name, binary_name, threads, "aborted", e.returncode, flush=True)
                        continue
                for r in res["rows"]:
                    if r[0] == "":
                        r[0] = "START"
                entry.update({"rows": res["rows"], "vertex_sha256": sha(res["vertex"]),
                              "graph_sha256": sha(res["graph"]), "last": res["last"], "aborted": False})
                out.append(entry)
                print(name, binary_name, threads, len(res["rows"]), "rows", res["rows"][-2][0], flush=True)
    (HERE / "order_variants.json").write_text(json.dumps(out, indent=1))


def constraints():
    # A fixed tiny background graph: constraint generation ignores it.
    out = []
    base = REF_DATA / "test_1"
    for case in C.constraint_cases():
        p = C.make_pattern(case)
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            p.write(tmp / "pattern")
            res = run_reference(base / "graph.totem", base / "vertex_data" / "graph_vertex_data.totem",
                                tmp / "pattern", tmp / "out", timeout=60)
        out.append({"case": case, "dump": constraint_section(res["log"])})
    with gzip.open(HERE / "constraints.json.gz", "wt") as f:
        json.dump(out, f)
    print("constraint cases", len(out))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--skip-big", action="store_true", help="skip the scale-16 case (minutes of CPU)")
    ap.add_argument("--only", choices=["fixtures", "synthetic", "constraints", "big", "stream15", "article", "order"])
    a = ap.parse_args()
    if not REF_BIN.exists():
        sys.exit("build the reference first: make -C oracle ref")
    if a.only in (None, "fixtures"):
        fixtures()
    if a.only in (None, "constraints"):
        constraints()
    if a.only in (None, "synthetic"):
        synthetic(True)
    if a.only in (None, "big") and not a.skip_big:
        synthetic(False, only_big=True)
    if a.only == "stream15":
        stream15()
    if a.only == "article":
        article()
    if a.only == "order":
        order()
