"""Dataset tooling: the reference's `toolset/` programs that turn an edge
list into the on-disk CSR and decorate it (the steps of `prepare_data.sh`).

  EdgeList2CSR <in dir> <out dir> [skip char]   toolset/edgelist_to_csr.cpp:6-42
  AssignWeight <dir> <lower> <upper> [seed]     toolset/assign_weight.cpp:18-52
  AssignEdgeLabel <dir> <labels> [seed]         toolset/assign_edge_label.cpp:16-44

Run as ``python -m thunderrw_gb300.toolset <Tool> ...``.

EdgeList2CSR reads ``<in dir>/b_edge_list.bin``, a text file of ``src dst``
lines (lines starting with the skip character are comments), and builds the
CSR exactly as Graph::load_edge_list does (graph.cpp:426-519): every edge is
taken as (min, max), pairs are sorted and deduplicated, self loops dropped,
and each remaining pair is stored in both directions, so every neighbour
list comes out sorted and free of repeats; n = largest id + 1.

The reference assigns weights and labels from ``std::random_device`` (a new
graph every run); these take a seed and draw from numpy's PCG64, one value
per directed CSR entry as the reference does (so w(u, v) and w(v, u) are
independent draws).
"""
from __future__ import annotations

import os
import sys

import numpy as np

from . import formats

EDGE_LIST = "b_edge_list.bin"  # graph.cpp:25 (a text file despite its name)


def read_edge_list(path: str, skip: str = "#") -> np.ndarray:
    """Graph::load_edge_list (graph.cpp:426-455): int64 [m, 2] of (min, max)
    pairs in file order."""
    rows = []
    with open(path, "r") as f:
        for lineno, line in enumerate(f, 1):
            if not line.strip() or line[0] == skip:
                continue
            parts = line.split()
            if len(parts) < 2:
                raise ValueError("cannot convert line %d to an edge" % lineno)
            rows.append((int(parts[0]), int(parts[1])))
    e = np.array(rows, dtype=np.int64).reshape(-1, 2)
    if e.size and e.min() < 0:
        raise ValueError("negative vertex id")
    return np.sort(e, axis=1)


def edges_to_csr(pairs: np.ndarray, num_vertices: int | None = None):
    """CSR of the undirected simple graph on (min, max) pairs
    (graph.cpp:463-519): returns (row int64 [n+1], adj int32 [e])."""
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    n = int(pairs.max()) + 1 if pairs.size else 0
    if num_vertices is not None:
        n = max(n, int(num_vertices))
    u, v = pairs[:, 0], pairs[:, 1]
    keep = u != v
    key = np.unique(u[keep] * max(n, 1) + v[keep])  # sorted, deduplicated (min, max) pairs
    u, v = key // max(n, 1), key % max(n, 1)
    src = np.concatenate([u, v])
    dst = np.concatenate([v, u])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    row = np.zeros(n + 1, dtype=np.int64)
    np.add.at(row, src + 1, 1)
    np.cumsum(row, out=row)
    if n > 0 and row[-1] >= (1 << 31):
        raise ValueError("%d CSR entries: the engine stores int32 offsets (< 2^31)" % row[-1])
    return row, dst.astype(np.int32)


def edgelist_to_csr(in_dir: str, out_dir: str, skip: str = "#"):
    """EdgeList2CSR: <in_dir>/b_edge_list.bin -> CSR files in <out_dir>."""
    row, adj = edges_to_csr(read_edge_list(os.path.join(in_dir, EDGE_LIST), skip))
    formats.store_csr(out_dir, row, adj)
    return row, adj


def _edges(graph_dir: str) -> int:
    with open(os.path.join(graph_dir, formats.DEGREE), "rb") as f:
        head = f.read(16)
    return int(np.frombuffer(head[8:16], np.int64)[0])


def assign_weight(graph_dir: str, lower: float, upper: float, seed: int = 0) -> np.ndarray:
    """AssignWeight: U[lower, upper) per CSR entry -> b_edge_weight.bin."""
    if not upper > lower:
        raise ValueError("upper bound must exceed the lower bound")
    w = np.random.default_rng(seed).uniform(lower, upper, _edges(graph_dir))
    w.astype(np.float64).tofile(os.path.join(graph_dir, formats.EDGE_WEIGHT))
    return w


def assign_edge_label(graph_dir: str, num_labels: int, seed: int = 0) -> np.ndarray:
    """AssignEdgeLabel: uniform labels in [0, num_labels) -> b_edge_label.bin."""
    if num_labels < 1:
        raise ValueError("need at least one label")
    lab = np.random.default_rng(seed).integers(0, num_labels, _edges(graph_dir), dtype=np.int32)
    lab.tofile(os.path.join(graph_dir, formats.EDGE_LABEL))
    return lab


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    tools = {"EdgeList2CSR": 2, "AssignWeight": 3, "AssignEdgeLabel": 2}
    if not argv or argv[0] not in tools or len(argv) - 1 < tools[argv[0]]:
        sys.stderr.write("usage: python -m thunderrw_gb300.toolset EdgeList2CSR <in dir> <out dir> [skip char]\n"
                         "       python -m thunderrw_gb300.toolset AssignWeight <dir> <lower> <upper> [seed]\n"
                         "       python -m thunderrw_gb300.toolset AssignEdgeLabel <dir> <labels> [seed]\n")
        return 2
    tool, a = argv[0], argv[1:]
    if tool == "EdgeList2CSR":
        row, adj = edgelist_to_csr(a[0], a[1], a[2][0] if len(a) > 2 else "#")
        print("|V| = %d, |E| = %d" % (row.size - 1, adj.size))
    elif tool == "AssignWeight":
        assign_weight(a[0], float(a[1]), float(a[2]), int(a[3]) if len(a) > 3 else 0)
    else:
        assign_edge_label(a[0], int(a[1]), int(a[2]) if len(a) > 2 else 0)
    return 0


if __name__ == "__main__":
    sys.exit(main())
