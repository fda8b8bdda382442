"""TOTEM file formats, seeded generators and the C ABI symbol table (CPU)."""
import re
import struct
from pathlib import Path

import numpy as np
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from tests import pmtest

ROOT = Path(__file__).resolve().parents[1]
DATA = pmtest.GOLDEN / "data"


def _parse_text(path):
    lines = [l for l in Path(path).read_text().splitlines() if l.strip()]
    V = int(lines[0].split(":")[1])
    E = int(lines[1].split(":")[1])
    edges = [tuple(map(int, l.split()[:2])) for l in lines[3:] if not l.startswith("#")]
    off = np.zeros(V + 1, np.uint64)
    for s, _ in edges:
        off[s + 1] += 1
    return V, E, np.cumsum(off).astype(np.uint64), np.array([d for _, d in edges], np.uint32)


@pytest.mark.parametrize("name", ["test_1", "test_2", "test_4"])
def test_text_reader_matches_plain_parse(name):
    g = pm.Graph.load(DATA / name / "graph.totem", None, DATA / name / "vertex_data" / "graph_vertex_data.totem",
                      device=-1)
    V, E, off, adj = _parse_text(DATA / name / "graph.totem")
    o, a, lab = g.host_csr()
    assert g.vertex_count == V and g.edge_count == E
    assert np.array_equal(o, off) and np.array_equal(a, adj)
    labels = dict(tuple(map(int, l.split())) for l in
                  (DATA / name / "vertex_data" / "graph_vertex_data.totem").read_text().split("\n") if l.strip())
    assert [int(x) for x in lab] == [labels.get(v, 0) for v in range(V)]


def test_binary_fixture_reads():
    # test_3/graph.totem is in TOTEM's binary format (magic 0x10102048)
    raw = (DATA / "test_3" / "graph.totem").read_bytes()
    assert struct.unpack("<I", raw[:4])[0] == 0x10102048
    g = pm.Graph.load(DATA / "test_3" / "graph.totem", None, None, device=-1)
    assert g.vertex_count == 12 and g.edge_count == 32


def test_binary_round_trip(tmp_path):
    g = pm.Graph.rmat(8, 8, seed=3).assign_labels("uniform", 4, seed=2)
    g.store_binary(tmp_path / "g.bin")
    h = pm.Graph.load(tmp_path / "missing.totem", tmp_path / "g.bin", None, device=-1)
    for x, y in zip(g.host_csr(), h.host_csr()):
        assert np.array_equal(x, y)


def test_text_round_trip(tmp_path):
    g = pm.Graph.rmat(7, 4, seed=5).assign_labels("zipf", 5, 1.0, seed=1)
    g.write_text(tmp_path / "g.totem", tmp_path / "l.totem")
    h = pm.Graph.load(tmp_path / "g.totem", None, tmp_path / "l.totem", device=-1)
    for x, y in zip(g.host_csr(), h.host_csr()):
        assert np.array_equal(x, y)


def test_bin_cache_replaces_text_and_labels(tmp_path):
    # multiple_label_cpu.cc:23: an existing .bin is loaded instead of the text
    # graph and its label file.
    g = pm.Graph.rmat(6, 4, seed=1).assign_labels("uniform", 3, seed=1)
    g.write_text(tmp_path / "g.totem", tmp_path / "l.totem")
    first = pm.Graph.load(tmp_path / "g.totem", tmp_path / "g.bin", tmp_path / "l.totem", device=-1)
    assert (tmp_path / "g.bin").exists()
    (tmp_path / "l2.totem").write_text("".join(f"{v} 9\n" for v in range(first.vertex_count)))
    second = pm.Graph.load(tmp_path / "g.totem", tmp_path / "g.bin", tmp_path / "l2.totem", device=-1)
    assert np.array_equal(first.host_csr()[2], second.host_csr()[2])


@pytest.mark.parametrize("content,code", [
    ("#Nodes:3\n#Edges:4\n#Undirected\n0 1\n1 0\n", pm.PM_E_FORMAT),            # truncated edge list
    ("#Nodes:3\n#Edges:2\n#Undirected\n1 0\n0 1\n", pm.PM_E_FORMAT),            # not sorted by source
    ("#Nodes:3\n#Undirected\n0 1\n", pm.PM_E_FORMAT),                            # missing EDGES line
    ("Nodes:3\n#Edges:2\n#Undirected\n0 1\n1 0\n", pm.PM_E_FORMAT),              # header without '#'
    ("#Nodes:3\n#Edges:2\n#Undirected\n0 x\n1 0\n", pm.PM_E_FORMAT),             # non-numeric id
    ("#Nodes:2\n#Edges:1\n#Undirected\n0 5\n", pm.PM_E_FORMAT),                  # target out of range
])
def test_malformed_text_rejected(tmp_path, content, code):
    p = tmp_path / "bad.totem"
    p.write_text(content)
    with pytest.raises(pm.PmError) as e:
        pm.Graph.load(p, None, None, device=-1)
    assert e.value.code == code


def test_truncated_binary_rejected(tmp_path):
    g = pm.Graph.rmat(6, 4, seed=2)
    g.store_binary(tmp_path / "g.bin")
    raw = (tmp_path / "g.bin").read_bytes()
    (tmp_path / "t.bin").write_bytes(raw[: len(raw) // 2])
    with pytest.raises(pm.PmError) as e:
        pm.Graph.load(tmp_path / "t.bin", None, None, device=-1)
    assert e.value.code == pm.PM_E_FORMAT


def test_missing_file():
    with pytest.raises(pm.PmError) as e:
        pm.Graph.load("/nonexistent/graph.totem", None, None, device=-1)
    assert e.value.code == pm.PM_E_IO


def test_rmat_properties_and_determinism():
    a = pm.Graph.rmat(10, 16, seed=7)
    b = pm.Graph.rmat(10, 16, seed=7)
    oa, aa, _ = a.host_csr()
    ob, ab, _ = b.host_csr()
    assert np.array_equal(oa, ob) and np.array_equal(aa, ab)
    V = a.vertex_count
    src = np.repeat(np.arange(V), np.diff(oa.astype(np.int64)))
    assert not np.any(src == aa), "self loops"
    for v in range(V):
        nb = aa[oa[v]:oa[v + 1]]
        assert np.all(np.diff(nb.astype(np.int64)) > 0), "adjacency must be strictly increasing"
    pairs = set(zip(src.tolist(), aa.tolist()))
    assert all((d, s) in pairs for s, d in pairs), "graph must be symmetric"


def test_label_kinds():
    g = pm.Graph.rmat(10, 8, seed=1).assign_labels("zipf", 16, 1.0, seed=3)
    lab = g.host_csr()[2]
    counts = np.bincount(lab.astype(np.int64), minlength=16)
    assert counts[0] > counts[15] and lab.max() < 16
    g2 = pm.Graph.rmat(10, 8, seed=1).assign_labels("degree", 8, 1.2, seed=3)
    assert g2.host_csr()[2].max() < 8


def _declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(pm_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.mark.parametrize("name", _declared_functions())
def test_library_exports_declared_symbol(name):
    assert hasattr(pm.lib, name), f"{name} declared in include/ but not exported"


def test_version_and_last_error():
    assert "sm_103a" in pm.version()
    with pytest.raises(pm.PmError):
        pm.Graph.load("/nonexistent", None, None, device=-1)
    assert "nonexistent" in pm.lib.pm_last_error().decode()


def _c_struct_fields(header: str, name: str) -> list[str]:
    """Field names of `typedef struct name {...} name;` in an include/ header, in order."""
    text = (Path(__file__).resolve().parent.parent / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", text, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        names = decl.split(None, 1)[1] if decl.split()[0] != "const" else decl.split(None, 2)[2]
        fields += [n.strip().lstrip("*").split("[")[0] for n in names.split(",")]
    return fields


@pytest.mark.parametrize("header,c_name,py_cls", [
    ("pm_gb300_tools.h", "pm_tune_result", "TuneResult"),
    ("pm_gb300.h", "pm_server_config", "ServerConfig"),
    ("pm_gb300.h", "pm_request_result", "RequestResult"),
    ("pm_gb300.h", "pm_server_stats", "ServerStats"),
])
def test_python_structs_mirror_the_header(header, c_name, py_cls):
    """The ctypes mirrors list the C structs' fields in the same order."""
    import ctypes

    cls = getattr(pm, py_cls)
    assert [n for n, _ in cls._fields_] == _c_struct_fields(header, c_name)
    assert all(ctypes.sizeof(t) in (4, 8) for _, t in cls._fields_)
