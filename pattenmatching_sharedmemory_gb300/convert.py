"""Input converters of the reference's pattern-matching scripts
(src/scripts/patternmatching/convert_edges2totem.py, crunch_vertex_data.py):
plain file transforms that produce the TOTEM text graph and the vertex label
file the pipeline reads.

    python -m pattenmatching_sharedmemory_gb300.convert edges2totem -i edges -o graph.totem [-d]
    python -m pattenmatching_sharedmemory_gb300.convert vertex-data -i a.vertex_data b.vertex_data -o labels
"""
from __future__ import annotations

import argparse
import os
import shutil
from pathlib import Path

_CHUNK = 1 << 20


def _last_line(path: Path) -> bytes:
    """The file's last non-empty line (read backwards from the end)."""
    with open(path, "rb") as f:
        f.seek(0, os.SEEK_END)
        end = f.tell()
        pos, tail = end, b""
        while pos > 0:
            step = min(4096, pos)
            pos -= step
            f.seek(pos)
            tail = f.read(step) + tail
            lines = [x for x in tail.split(b"\n") if x.strip()]
            if len(lines) >= 2 or (lines and pos == 0):
                return lines[-1]
        return b""


def _line_count(path: Path) -> int:
    n = 0
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(_CHUNK), b""):
            n += chunk.count(b"\n")
    return n


def edges_to_totem(input_path, output_path, directed: bool = False) -> tuple[int, int]:
    """convert_edges2totem.py: a `src dst` edge list sorted by source becomes
    a TOTEM text graph.  As in the reference, the vertex count is the last
    line's source id + 1 and the edge count is the input's line count; the
    header is `#Nodes: V`, `#Edges: E`, `#Directed` or `#Undirected`, and
    the edge lines follow unchanged.  Returns (V, E)."""
    src, dst = Path(input_path), Path(output_path)
    last = _last_line(src)
    if not last:
        raise ValueError(f"{src}: no edge lines")
    nodes = int(last.split()[0]) + 1
    edges = _line_count(src)
    with open(src, "rb") as fin, open(dst, "wb") as fout:
        fout.write(f"#Nodes: {nodes}\n#Edges: {edges}\n".encode())
        fout.write(b"#Directed\n" if directed else b"#Undirected\n")
        shutil.copyfileobj(fin, fout, _CHUNK)
    return nodes, edges


def concat_vertex_data(input_paths, output_path) -> int:
    """crunch_vertex_data.py: `vid label` files (one per vertex class, each
    covering its own id range) concatenated, in the given order, into the
    single vertex label file the pipeline reads.  Returns the bytes written."""
    written = 0
    with open(output_path, "wb") as fout:
        for p in input_paths:
            with open(p, "rb") as fin:
                for chunk in iter(lambda: fin.read(_CHUNK), b""):
                    fout.write(chunk)
                    written += len(chunk)
    return written


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(prog="python -m pattenmatching_sharedmemory_gb300.convert")
    sub = ap.add_subparsers(dest="cmd", required=True)
    e = sub.add_parser("edges2totem", help="sorted `src dst` edge list -> TOTEM text graph")
    e.add_argument("-i", "--input", required=True)
    e.add_argument("-o", "--output", required=True)
    e.add_argument("-d", "--directed", action="store_true")
    v = sub.add_parser("vertex-data", help="concatenate `vid label` files")
    v.add_argument("-i", "--input-list", nargs="+", required=True)
    v.add_argument("-o", "--output", required=True)
    a = ap.parse_args(argv)
    if a.cmd == "edges2totem":
        n, m = edges_to_totem(a.input, a.output, a.directed)
        print(f"converted {a.input} into {a.output}: {n} vertices, {m} edge lines")
    else:
        b = concat_vertex_data(a.input_list, a.output)
        print(f"wrote {b} bytes to {a.output}")


if __name__ == "__main__":
    main()
