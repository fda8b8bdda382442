"""Template (query pattern) type and seeded template generators.

All randomness comes from splitmix64 on integers, so a seed gives the same
template on every machine.  Templates are connected, undirected, stored with
both edge directions and sorted adjacency, like the reference's
pattern_edge files (data/patternmatching/test_*/pattern_1/pattern_edge).

This module is plain numpy: it does not load the GPU library (only
Pattern.dump_constraints does, when called), so CPU-side callers can
generate the same template streams without it.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_MASK = (1 << 64) - 1


@dataclass
class Pattern:
    """A template graph in CSR form with per-vertex labels."""

    offsets: np.ndarray
    adj: np.ndarray
    labels: np.ndarray

    @property
    def n(self) -> int:
        return len(self.offsets) - 1

    @classmethod
    def from_edges(cls, n: int, edges, labels) -> "Pattern":
        """Undirected template from an edge list (both directions stored, sorted)."""
        nbrs = [set() for _ in range(n)]
        for u, v in edges:
            nbrs[u].add(v)
            nbrs[v].add(u)
        off = np.zeros(n + 1, np.uint64)
        adj = []
        for u in range(n):
            adj.extend(sorted(nbrs[u]))
            off[u + 1] = len(adj)
        return cls(off, np.asarray(adj, np.uint32), np.asarray(labels, np.uint64))

    def dump_constraints(self) -> str:
        """Reference-format constraint dump (log.totem) of this template
        (the template compiler of the GPU library)."""
        from . import _check, lib

        off = np.ascontiguousarray(self.offsets, np.uint64)
        adj = np.ascontiguousarray(self.adj, np.uint32)
        lab = np.ascontiguousarray(self.labels, np.uint64)
        args = (off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                adj.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                lab.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), self.n, len(adj))
        need = ctypes.c_size_t()
        _check(lib.pm_template_dump_constraints(*args, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        _check(lib.pm_template_dump_constraints(*args, buf, need.value, None))
        return buf.value.decode()

    def write(self, directory) -> None:
        """Writes pattern_edge (TOTEM text) and pattern_vertex_data."""
        d = Path(directory)
        d.mkdir(parents=True, exist_ok=True)
        lines = [f"#Nodes:{self.n}", f"#Edges:{len(self.adj)}", "#Undirected"]
        for u in range(self.n):
            for e in range(int(self.offsets[u]), int(self.offsets[u + 1])):
                lines.append(f"{u} {int(self.adj[e])}")
        (d / "pattern_edge").write_text("\n".join(lines) + "\n")
        (d / "pattern_vertex_data").write_text("".join(f"{u} {int(self.labels[u])}\n" for u in range(self.n)))


def splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & _MASK
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _MASK
    return x ^ (x >> 31)


class Rng:
    def __init__(self, seed: int):
        self.s = splitmix64(seed & _MASK)

    def next(self) -> int:
        self.s = splitmix64(self.s)
        return self.s

    def below(self, n: int) -> int:
        return (self.next() * n) >> 64

    def unit(self) -> float:
        return (self.next() >> 11) / float(1 << 53)


def cycle(labels) -> Pattern:
    n = len(labels)
    return Pattern.from_edges(n, [(i, (i + 1) % n) for i in range(n)], labels)


def two_cycles_sharing_edge(labels) -> Pattern:
    """Six vertices: 4-cycle 0-1-2-3 and 4-cycle 2-3-4-5 sharing edge (2,3)."""
    assert len(labels) == 6
    return Pattern.from_edges(6, [(0, 1), (1, 2), (2, 3), (3, 0), (3, 4), (4, 5), (5, 2)], labels)


def random_template(n: int, density: float, label_weights, seed: int, distinct: bool = False) -> Pattern:
    """Connected template with about density * n(n-1)/2 edges (at least a
    spanning tree); vertex labels drawn from label_weights (index = label),
    without repetition when distinct is set."""
    rng = Rng(seed)
    order = list(range(n))
    for i in range(n - 1, 0, -1):
        j = rng.below(i + 1)
        order[i], order[j] = order[j], order[i]
    edges = set()
    for i in range(1, n):
        u, v = order[i], order[rng.below(i)]
        edges.add((min(u, v), max(u, v)))
    target = max(n - 1, round(density * n * (n - 1) / 2))
    all_pairs = [(u, v) for u in range(n) for v in range(u + 1, n) if (u, v) not in edges]
    while len(edges) < target and all_pairs:
        edges.add(all_pairs.pop(rng.below(len(all_pairs))))
    weights = list(label_weights)
    labels = []
    for _ in range(n):
        total = sum(weights)
        r = rng.unit() * total
        acc = 0.0
        pick = len(weights) - 1
        for i, w in enumerate(weights):
            acc += w
            if r < acc:
                pick = i
                break
        labels.append(pick)
        if distinct:
            weights[pick] = 0.0
    return Pattern.from_edges(n, sorted(edges), labels)


def zipf_weights(n_labels: int, s: float):
    return [1.0 / (i + 1) ** s for i in range(n_labels)]


def served_stream(count: int, n_labels: int = 32, zipf_s: float = 1.2, seed: int = 24, min_vertices: int = 3,
                  max_vertices: int = 10, min_density: float = 0.3, max_density: float = 0.6) -> list:
    """The served workload's query stream: `count` seeded connected templates
    of min..max vertices and edge density min..max, vertex labels drawn from
    the graph's Zipf(zipf_s) label distribution over n_labels labels
    (repeats allowed, so template-driven search is exercised).  Template i
    depends only on (seed, i), so any prefix or sample of the stream is
    reproducible on its own."""
    weights = zipf_weights(n_labels, zipf_s)
    out = []
    for i in range(count):
        rng = Rng(splitmix64(seed * 0x100000001B3 + i))
        n = min_vertices + rng.below(max_vertices - min_vertices + 1)
        density = min_density + (max_density - min_density) * rng.unit()
        out.append(random_template(n, density, weights, seed=rng.next()))
    return out
