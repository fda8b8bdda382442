"""Seeded parity cases shared by the golden-fixture generator and the tests.

A case names a synthetic graph (RMAT generator + label assignment) and a
template; both are rebuilt deterministically from these parameters on any
machine, and the reference's outputs for them are stored in
tests/golden/synthetic_cases.json.
"""
from __future__ import annotations

from pathlib import Path

import pattenmatching_sharedmemory_gb300 as pm
from pattenmatching_sharedmemory_gb300 import templates as T

GOLDEN = Path(__file__).resolve().parent / "golden"

FIXTURE_PATTERNS = {
    # pattern_1 of the reference's bundled fixtures, as edge lists + labels
    "test_1": (3, [(0, 1), (0, 2), (1, 2)], [0, 1, 2]),
    "test_3": (4, [(0, 1), (0, 2), (0, 3), (1, 2), (2, 3)], [0, 1, 2, 1]),
    "test_4": (10, [(0, 1), (1, 2), (2, 3), (2, 6), (2, 8), (3, 4), (4, 5), (4, 6), (4, 7), (7, 8), (8, 9)],
               [1, 2, 3, 4, 2, 6, 5, 5, 6, 2]),
}


def graph_params(scale, ef=16, seed=1, kind="uniform", n_labels=5, s=1.0, label_seed=1, permute=True):
    return {"scale": scale, "ef": ef, "a": 0.57, "b": 0.19, "c": 0.19, "seed": seed, "permute": permute,
            "labels": {"kind": kind, "n": n_labels, "s": s, "seed": label_seed}}


def make_graph(case) -> pm.Graph:
    gp = case["graph"]
    g = pm.Graph.rmat(gp["scale"], gp["ef"], gp["a"], gp["b"], gp["c"], gp["seed"], gp["permute"])
    lp = gp["labels"]
    g.assign_labels(lp["kind"], lp["n"], lp["s"], lp["seed"])
    return g


def make_pattern(case) -> pm.Pattern:
    p = case["pattern"]
    if p["kind"] == "cycle":
        return T.cycle(p["labels"])
    if p["kind"] == "two_cycles":
        return T.two_cycles_sharing_edge(p["labels"])
    if p["kind"] == "edges":
        return pm.Pattern.from_edges(p["n"], [tuple(e) for e in p["edges"]], p["labels"])
    if p["kind"] == "fixture":
        n, edges, labels = FIXTURE_PATTERNS[p["name"]]
        return pm.Pattern.from_edges(n, edges, labels)
    if p["kind"] == "random":
        w = T.zipf_weights(p["label_n"], p.get("zipf_s", 0.0))
        return T.random_template(p["n"], p["density"], w, p["seed"], p.get("distinct", False))
    raise ValueError(p["kind"])


def synthetic_cases(include_big: bool = True):
    cases = []

    def add(name, graph, pattern, **kw):
        c = {"name": name, "graph": graph, "pattern": pattern}
        c.update(kw)
        cases.append(c)

    add("c1_scale10_cycle4", graph_params(10), {"kind": "cycle", "labels": [0, 1, 2, 3]})
    add("triangle_s9", graph_params(9, n_labels=3), {"kind": "cycle", "labels": [0, 1, 2]})
    add("triangle_rep_s9", graph_params(9, n_labels=2, label_seed=3), {"kind": "cycle", "labels": [0, 0, 1]})
    add("cycle4_rep_s9", graph_params(9, ef=8, n_labels=2, label_seed=4), {"kind": "cycle", "labels": [0, 1, 0, 1]})
    add("cycle5_s10", graph_params(10, n_labels=4, label_seed=5), {"kind": "cycle", "labels": [0, 1, 2, 3, 1]})
    add("path_rep_s9", graph_params(9, n_labels=3, label_seed=6),
        {"kind": "edges", "n": 3, "edges": [(0, 1), (1, 2)], "labels": [0, 1, 0]})
    add("path4_rep_s9", graph_params(9, n_labels=3, label_seed=7),
        {"kind": "edges", "n": 4, "edges": [(0, 1), (1, 2), (2, 3)], "labels": [1, 0, 2, 1]})
    add("star_s9", graph_params(9, n_labels=3, label_seed=8),
        {"kind": "edges", "n": 4, "edges": [(0, 1), (0, 2), (0, 3)], "labels": [0, 1, 1, 2]})
    add("fixture3_s9", graph_params(9, n_labels=3, label_seed=9), {"kind": "fixture", "name": "test_3"})
    add("fixture4_s10", graph_params(10, n_labels=7, label_seed=10), {"kind": "fixture", "name": "test_4"})
    add("fixture1_s10_zipf", graph_params(10, kind="zipf", n_labels=3, s=1.0, label_seed=11),
        {"kind": "fixture", "name": "test_1"})
    add("two_cycles_s10", graph_params(10, n_labels=6, label_seed=12),
        {"kind": "two_cycles", "labels": [0, 1, 2, 3, 4, 5]})
    add("two_cycles_zipf_s10", graph_params(10, kind="zipf", n_labels=16, s=1.0, label_seed=13),
        {"kind": "two_cycles", "labels": [0, 1, 2, 3, 4, 5]})
    add("degree_labels_s10", graph_params(10, kind="degree", n_labels=8, s=1.2, label_seed=14),
        {"kind": "cycle", "labels": [0, 1, 2, 3]})
    add("k4_rep_s8", graph_params(8, n_labels=2, label_seed=15),
        {"kind": "edges", "n": 4, "edges": [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)], "labels": [0, 1, 0, 1]})
    for i in range(16):
        n = 3 + i % 6
        add(f"random_{i:02d}", graph_params(8 + i % 3, ef=8 + 8 * (i % 2), n_labels=3 + i % 4, label_seed=100 + i),
            {"kind": "random", "n": n, "density": 0.3 + 0.1 * (i % 4), "label_n": 3 + i % 4, "zipf_s": 0.0,
             "seed": 1000 + i, "distinct": i % 3 == 0})
    add("scale12_cycle4", graph_params(12, n_labels=5, label_seed=2), {"kind": "cycle", "labels": [0, 1, 2, 3]})
    add("scale12_tds", graph_params(12, kind="zipf", n_labels=8, s=1.0, label_seed=3),
        {"kind": "random", "n": 6, "density": 0.5, "label_n": 8, "zipf_s": 1.0, "seed": 77})
    if include_big:
        add("c1_scale16_cycle4", graph_params(16), {"kind": "cycle", "labels": [0, 1, 2, 3]}, ref_threads=1,
            timeout=14400, big=True)
    return cases


def stream15_cases():
    """The served RMAT-16 stream: the 15 4-cycles with four distinct labels
    of 0..4 (every 4-subset in its 3 cyclic orders), full pipeline.  The
    reference runs them with several threads (hours of CPU at one thread);
    for distinct labels no memo test can block a walk, so the outputs do not
    depend on the thread count."""
    import itertools

    cases = []
    for a, b, c, d in itertools.combinations(range(5), 4):
        for order in ([a, b, c, d], [a, b, d, c], [a, c, b, d]):
            cases.append({"name": "stream15_" + "".join(map(str, order)), "graph": graph_params(16),
                          "pattern": {"kind": "cycle", "labels": list(order)}, "ref_threads": 5, "timeout": 7200,
                          "big": True})
    return cases


def constraint_cases():
    cases = []
    for name in FIXTURE_PATTERNS:
        cases.append({"name": f"fixture_{name}", "pattern": {"kind": "fixture", "name": name}})
    shapes = {
        "k4": (4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]),
        "k5": (5, [(i, j) for i in range(5) for j in range(i + 1, 5)]),
        "wheel5": (6, [(0, i) for i in range(1, 6)] + [(i, i % 5 + 1) for i in range(1, 6)]),
        "path6": (6, [(i, i + 1) for i in range(5)]),
        "star6": (6, [(0, i) for i in range(1, 6)]),
        "two_triangles": (5, [(0, 1), (1, 2), (2, 0), (2, 3), (3, 4), (4, 2)]),
    }
    for name, (n, edges) in shapes.items():
        for li, labels in enumerate([list(range(n)), [i % 2 for i in range(n)], [i % 3 for i in range(n)], [0] * n]):
            cases.append({"name": f"{name}_{li}", "pattern": {"kind": "edges", "n": n, "edges": edges,
                                                              "labels": labels}})
    for i in range(130):
        n = 3 + i % 7
        cases.append({"name": f"random_{i:03d}",
                      "pattern": {"kind": "random", "n": n, "density": 0.2 + 0.1 * (i % 6), "label_n": 2 + i % 4,
                                  "zipf_s": 0.0, "seed": 5000 + i, "distinct": False}})
    return cases
