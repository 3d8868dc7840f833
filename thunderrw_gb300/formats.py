"""The reference's on-disk CSR format (util/graph/graph.cpp:18-30, 123-212,
233-287): one directory holding

  b_degree.bin                    u32 element size (4), i32 n, i64 e, then n i32 degrees
                                  (graph.cpp:138-144 writes, :238-247 reads)
  b_adj.bin                       e i32 neighbour ids
  b_edge_weight.bin               e f64 edge weights
  b_edge_label.bin                e i32 edge labels
  b_edge_weight_prefix_sum.bin    e f64 ITS prefix sums
  b_edge_weight_alias_table.bin   e x 16-byte AliasSlot {f64 prob, i32 first, i32 second}
  b_edge_weight_max.bin           n f64 rejection maxima

so graphs and tables move between the reference binaries and this engine.
"""
from __future__ import annotations

import os

import numpy as np

ALIAS_DTYPE = np.dtype([("prob", "<f8"), ("first", "<i4"), ("second", "<i4")])

DEGREE = "b_degree.bin"
ADJ = "b_adj.bin"
EDGE_WEIGHT = "b_edge_weight.bin"
EDGE_LABEL = "b_edge_label.bin"
PREFIX = "b_edge_weight_prefix_sum.bin"
ALIAS = "b_edge_weight_alias_table.bin"
MAX = "b_edge_weight_max.bin"


def _np(x, dtype):
    if x is None:
        return None
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


def store_csr(graph_dir: str, row, adj, weight=None, label=None, prefix=None, alias=None, rmax=None):
    """Graph::store_csr (graph.cpp:123-212)."""
    os.makedirs(graph_dir, exist_ok=True)
    row = _np(row, np.int64)
    adj = _np(adj, np.int32)
    n, e = row.size - 1, adj.size
    deg = np.diff(row).astype(np.int32)
    with open(os.path.join(graph_dir, DEGREE), "wb") as f:
        f.write(np.uint32(4).tobytes())
        f.write(np.int32(n).tobytes())
        f.write(np.int64(e).tobytes())
        f.write(deg.tobytes())
    adj.tofile(os.path.join(graph_dir, ADJ))
    for arr, name, dt in ((weight, EDGE_WEIGHT, np.float64), (label, EDGE_LABEL, np.int32),
                          (prefix, PREFIX, np.float64), (rmax, MAX, np.float64)):
        if arr is not None:
            _np(arr, dt).tofile(os.path.join(graph_dir, name))
    if alias is not None:
        np.ascontiguousarray(alias, dtype=ALIAS_DTYPE).tofile(os.path.join(graph_dir, ALIAS))


def load_csr(graph_dir: str, edge_weight=False, edge_label=False, prefix=False, alias=False, rmax=False):
    """Graph::load_csr (graph.cpp:45-101): degree file -> offsets, then the
    optional per-edge / per-vertex arrays."""
    with open(os.path.join(graph_dir, DEGREE), "rb") as f:
        head = f.read(16)
        elem = int(np.frombuffer(head[:4], np.uint32)[0])
        if elem != 4:
            raise ValueError("b_degree.bin element size %d: only 4-byte vertex ids are supported" % elem)
        n = int(np.frombuffer(head[4:8], np.int32)[0])
        e = int(np.frombuffer(head[8:16], np.int64)[0])
        deg = np.frombuffer(f.read(4 * n), np.int32)
    if deg.size != n:
        raise ValueError("truncated b_degree.bin")
    row = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg, out=row[1:])
    if row[-1] != e:
        raise ValueError("degree sum %d != e %d" % (row[-1], e))
    out = {"n": n, "e": e, "row": row,
           "adj": np.fromfile(os.path.join(graph_dir, ADJ), dtype=np.int32, count=e)}
    if out["adj"].size != e:
        raise ValueError("truncated b_adj.bin")
    if edge_weight:
        out["weight"] = np.fromfile(os.path.join(graph_dir, EDGE_WEIGHT), dtype=np.float64, count=e)
    if edge_label:
        out["label"] = np.fromfile(os.path.join(graph_dir, EDGE_LABEL), dtype=np.int32, count=e)
    if prefix:
        out["prefix"] = np.fromfile(os.path.join(graph_dir, PREFIX), dtype=np.float64, count=e)
    if alias:
        out["alias"] = np.fromfile(os.path.join(graph_dir, ALIAS), dtype=ALIAS_DTYPE, count=e)
    if rmax:
        out["rmax"] = np.fromfile(os.path.join(graph_dir, MAX), dtype=np.float64, count=n)
    return out
