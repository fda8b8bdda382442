"""Graph ingestion tools (CPU): the TOTEM generator's UNDIRECTED,
SORT_NEIGHBOURS and SORT_VERTICES commands, against a restatement of the
generator's steps (src/generator/totem_generator.cc): every CSR entry
doubled, lists built from the edge list with each entry at the last free
position of its source's list (edgelist_to_graph, :92-125), ids renumbered
by ascending degree with ties by old id."""
from __future__ import annotations

import numpy as np

import pattenmatching_sharedmemory_gb300 as pm


def _edgelist_to_csr(src, dst, V):
    deg = np.bincount(np.asarray(src, np.int64), minlength=V)
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    adj = np.zeros(int(off[-1]), np.uint32)
    fill = deg.copy()
    for u, v in zip(src, dst):
        fill[u] -= 1
        adj[int(off[u]) + fill[u]] = v
    return off, adj


def _graph():
    rng = np.random.default_rng(5)
    V = 40
    src = rng.integers(0, V, 150)
    dst = rng.integers(0, V, 150)
    order = np.argsort(src, kind="stable")
    src, dst = src[order], dst[order]
    off = np.concatenate([[0], np.cumsum(np.bincount(src, minlength=V))]).astype(np.uint64)
    labels = rng.integers(0, 4, V).astype(np.uint64)
    return pm.Graph.from_csr(off, dst.astype(np.uint32), labels, device=-1), off, dst.astype(np.uint32), labels


def test_undirected_doubles_every_entry():
    g, off, adj, lab = _graph()
    u = g.undirected()
    V = len(off) - 1
    src, dst = [], []
    for v in range(V):
        for e in range(int(off[v]), int(off[v + 1])):
            src += [v, int(adj[e])]
            dst += [int(adj[e]), v]
    w_off, w_adj = _edgelist_to_csr(src, dst, V)
    o2, a2, l2 = u.host_csr()
    assert np.array_equal(o2, w_off) and np.array_equal(a2, w_adj) and np.array_equal(l2, lab)
    assert u.edge_count == 2 * g.edge_count


def test_sort_neighbours_in_place():
    g, off, adj, _ = _graph()
    u = g.undirected().sort_neighbours()
    o2, a2, _ = u.host_csr()
    for v in range(len(o2) - 1):
        seg = a2[int(o2[v]):int(o2[v + 1])]
        assert np.all(seg[:-1] <= seg[1:])


def test_sort_vertices_by_degree():
    g, off, adj, lab = _graph()
    s, m = g.sorted_by_degree()
    V = len(off) - 1
    deg = np.diff(off.astype(np.int64))
    order = np.argsort(deg, kind="stable")
    want_map = np.empty(V, np.uint32)
    want_map[order] = np.arange(V, dtype=np.uint32)
    assert np.array_equal(m, want_map)
    src, dst = [], []
    for v in range(V):
        for e in range(int(off[v]), int(off[v + 1])):
            src.append(int(want_map[v]))
            dst.append(int(want_map[adj[e]]))
    w_off, w_adj = _edgelist_to_csr(src, dst, V)
    o2, a2, l2 = s.host_csr()
    assert np.array_equal(o2, w_off) and np.array_equal(a2, w_adj)
    assert np.all(np.diff(np.diff(o2.astype(np.int64))) >= 0)  # degrees ascend
    assert np.array_equal(l2[want_map], lab)


def test_edges_to_totem_and_vertex_data(tmp_path):
    """The reference's converter scripts (src/scripts/patternmatching/
    convert_edges2totem.py, crunch_vertex_data.py): a sorted edge list gains
    the TOTEM header (vertex count = last line's source + 1, edge count =
    line count) and loads as the same CSR; vertex label files concatenate
    into one label file."""
    from pattenmatching_sharedmemory_gb300 import convert

    _, off, adj, lab = _graph()
    V = len(off) - 1
    last = max(u for u in range(V) if off[u + 1] > off[u])
    src = np.repeat(np.arange(V), np.diff(off.astype(np.int64)))
    edges = tmp_path / "edges"
    edges.write_text("".join(f"{u} {w}\n" for u, w in zip(src.tolist(), adj.tolist())))
    n, m = convert.edges_to_totem(edges, tmp_path / "graph.totem", directed=True)
    assert (n, m) == (last + 1, len(adj))
    head = (tmp_path / "graph.totem").read_text().splitlines()[:3]
    assert head == [f"#Nodes: {last + 1}", f"#Edges: {len(adj)}", "#Directed"]
    parts = [tmp_path / "a.vertex_data", tmp_path / "b.vertex_data"]
    half = (last + 1) // 2
    parts[0].write_text("".join(f"{v} {int(lab[v])}\n" for v in range(half)))
    parts[1].write_text("".join(f"{v} {int(lab[v])}\n" for v in range(half, last + 1)))
    convert.concat_vertex_data(parts, tmp_path / "labels")
    g = pm.Graph.load(tmp_path / "graph.totem", None, tmp_path / "labels", device=-1)
    o2, a2, l2 = g.host_csr()
    assert np.array_equal(o2, off[:last + 2]) and np.array_equal(a2, adj)
    assert np.array_equal(l2, lab[:last + 1])
    n, _ = convert.edges_to_totem(edges, tmp_path / "u.totem")
    assert (tmp_path / "u.totem").read_text().splitlines()[2] == "#Undirected"
