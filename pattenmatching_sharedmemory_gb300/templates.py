"""Seeded template (query pattern) generators.

All randomness comes from splitmix64 on integers, so a seed gives the same
template on every machine.  Templates are connected, undirected, stored with
both edge directions and sorted adjacency, like the reference's
pattern_edge files (data/patternmatching/test_*/pattern_1/pattern_edge).
"""
from __future__ import annotations

from . import Pattern

_MASK = (1 << 64) - 1


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
