"""Helpers shared by the tests: running the product and the oracle on a case
and rendering pruned state in the reference's output formats."""
from __future__ import annotations

import gzip
import hashlib
import json
import tempfile
from pathlib import Path

import numpy as np

import pattenmatching_sharedmemory_gb300 as pm
from tests import cases as C

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_fixture_golden():
    return json.loads((GOLDEN / "expected_fixtures.json").read_text())


def load_synthetic_golden():
    cases = json.loads((GOLDEN / "synthetic_cases.json").read_text())
    big = GOLDEN / "synthetic_big.json"
    if big.exists():
        cases += json.loads(big.read_text())
    return cases


def load_constraint_golden():
    with gzip.open(GOLDEN / "constraints.json.gz", "rt") as f:
        return json.load(f)


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def vertex_text(cand: np.ndarray, vact: np.ndarray) -> bytes:
    """vertex_NNNN.totem (MultipleLabelCpu::printActiveVertex, multiple_label_cpu.cc:286-296)."""
    out = []
    for v in np.nonzero(vact)[0]:
        c = int(cand[v])
        roles = "".join(f"{p} " for p in range(64) if c >> p & 1)
        out.append(f"{v} {roles}\n")
    return ("".join(out) + "\n").encode()


def graph_text(offsets, adj, labels, eact, vact) -> bytes:
    """graph_NNNN.totem (MultipleLabelCpu::printActiveGraph, multiple_label_cpu.cc:270-284)."""
    V = len(offsets) - 1
    deg = np.diff(offsets.astype(np.int64))
    src = np.repeat(np.arange(V, dtype=np.int64), deg)
    dst = adj.astype(np.int64)
    keep = (eact != 0) & (vact[src] != 0) & (vact[dst] != 0)
    s, d = src[keep], dst[keep]
    lab = labels.astype(np.uint64)
    lines = [f"{a} {b} {lab[a]} {lab[b]}\n" for a, b in zip(s.tolist(), d.tolist())]
    return ("".join(lines) + "\n").encode()


def oracle_case(case, threads=1):
    from oracle import oracle

    g = C.make_graph(case)
    off, adj, lab = g.host_csr()
    p = C.make_pattern(case)
    r = oracle.run(off, adj, lab, p.offsets, p.adj, p.labels, threads=threads)
    return g, r


def product_run(graph: pm.Graph, pattern=None, pattern_dir=None):
    """Runs the GPU pipeline and returns rows, output files and the query."""
    q = pm.Query(graph, pattern_dir=pattern_dir, pattern=pattern)
    recs = q.run()
    with tempfile.TemporaryDirectory() as tmp:
        q.write_outputs(tmp)
        last = recs[-1].iteration
        vtx = (Path(tmp) / f"vertex_{last:04d}.totem").read_bytes()
        grp = (Path(tmp) / f"graph_{last:04d}.totem").read_bytes()
        res = (Path(tmp) / "results.totem").read_text()
    rows = [list(r.as_tuple()) for r in recs]
    return {"rows": rows, "vertex": vtx, "graph": grp, "last": last, "results": res, "query": q, "records": recs}


def device_u64(a):
    """A uint64 / uint32 numpy array as a CUDA tensor (same bytes)."""
    import torch

    signed = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32}[a.dtype]
    return torch.from_numpy(np.ascontiguousarray(a).view(signed)).to("cuda:0")


def edge_bits(eact: np.ndarray) -> np.ndarray:
    """Per-CSR-entry flags -> one bit per entry, bit e % 32 of word e // 32."""
    b = np.packbits(eact.astype(np.uint8) != 0, bitorder="little")
    buf = np.zeros(max((len(eact) + 31) // 32, 1) * 4, np.uint8)
    buf[:len(b)] = b
    return buf.view("<u4").astype(np.uint32)


def sampled_count_gpu(graph, pattern, cand, eact, start_role: int, stride: int, residue: int = 0) -> int:
    """ENUMERATION count over the sources v % stride == residue only: the
    pruned state with the start role cleared on every other vertex, counted
    by pm_enumerate_noalloc (the start role is bound at the walk's first step
    only, so this is the per-source sum over the sampled sources)."""
    import ctypes

    import torch

    off, adj, _ = graph.host_csr()
    c = cand.copy()
    keep = (np.arange(len(c)) % stride) == residue
    c[~keep] &= ~np.uint64(1 << start_role)
    d_off, d_adj = device_u64(off.copy()), device_u64(adj.copy())
    d_cand, d_eact = device_u64(c), device_u64(edge_bits(eact))
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    po = np.ascontiguousarray(pattern.offsets, np.uint64)
    pa = np.ascontiguousarray(pattern.adj, np.uint32)
    pl = np.ascontiguousarray(pattern.labels, np.uint64)
    st = pm.lib.pm_enumerate_noalloc(d_off.data_ptr(), d_adj.data_ptr(), graph.vertex_count, graph.edge_count, 1,
                                     d_cand.data_ptr(), d_eact.data_ptr(),
                                     po.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                     pa.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                     pl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), pattern.n, len(pa),
                                     d_count.data_ptr(), None)
    if st != pm.PM_SUCCESS:
        raise pm.PmError(st, pm.lib.pm_last_error().decode())
    return int(d_count.item())
