"""Algorithmic bytes per step of each walk kernel, for the roofline.

Every independent random access is charged the 32-byte sectors it spans, a
contiguous row scan the sectors it spans, a path entry 4 bytes (written
step-major by consecutive steps of one walker).  The figures follow the
GPU kernels' methods:

  uniform move + PPR counts   row pair 32 + adjacency entry 32 + count 32
  static alias (DeepWalk)     row pair 32 + alias slot 32 + path 4
  Node2Vec (max-weight RS)    row pair 32 + candidate 32 + one probe of the
                              edge set 32 (not on the first move nor for a
                              return to the previous vertex) + path 4, per
                              accepted move; rejected trials are not charged,
                              so the figure is a lower bound
  MetaPath (dynamic ITS)      row pair 32 + the label row's sectors +
                              selected adjacency entry 32 + path 4 (row scan);
                              with the label index: row pair 32 + the two
                              label offsets 32 + the sorted neighbour 32 +
                              path 4

The per-walk figures are computed from the paths the GPU produced, so they
describe the same walks that were timed.
"""
from __future__ import annotations

import numpy as np

SECTOR = 32
UNIFORM_PPR = 96
STATIC_ALIAS = 68


def _span_sectors(begin_byte: np.ndarray, end_byte: np.ndarray) -> np.ndarray:
    """Sectors spanned by [begin, end) byte ranges (0 for empty ranges)."""
    nonempty = end_byte > begin_byte
    first = begin_byte // SECTOR
    last = (np.maximum(end_byte, begin_byte + 1) - 1) // SECTOR
    return np.where(nonempty, last - first + 1, 0)


def _moves(paths: np.ndarray):
    """(from, to, step index) of every recorded move: path entries k-1 -> k."""
    paths = np.asarray(paths)
    frm, to = paths[:, :-1], paths[:, 1:]
    valid = (frm >= 0) & (to >= 0)
    k = np.broadcast_to(np.arange(1, paths.shape[1]), frm.shape)
    return frm[valid], to[valid], k[valid], paths


def _stops(paths: np.ndarray, length: int):
    """Last vertex of every walk that stopped before `length` entries (a
    vertex without neighbours, or a row whose weights are all zero)."""
    n_entries = (np.asarray(paths) >= 0).sum(axis=1)
    early = (n_entries > 0) & (n_entries < length)
    return np.asarray(paths)[early, n_entries[early] - 1]


def node2vec(paths: np.ndarray, length: int) -> float:
    """Bytes per move of Node2Vec walks with the edge-set neighbour test
    (walks that stop early are charged the row pair of their last vertex)."""
    frm, to, k, p = _moves(paths)
    if frm.size == 0:
        return 0.0
    # previous vertex of each move: path entry k-2 (none for the first move)
    prev = np.full(p[:, :-1].shape, -1, dtype=np.int64)
    prev[:, 1:] = p[:, :-2]
    valid = (p[:, :-1] >= 0) & (p[:, 1:] >= 0)
    prev = prev[valid]
    probe = (k >= 2) & (to != prev)
    total = frm.size * (SECTOR + SECTOR + 4) + int(probe.sum()) * SECTOR + _stops(p, length).size * SECTOR
    return total / frm.size


def metapath(paths: np.ndarray, row: np.ndarray, length: int) -> float:
    """Bytes per move of MetaPath walks (label row scan per step; a walk that
    stops early is charged the row pair and label scan of its last vertex)."""
    frm, to, k, p = _moves(paths)
    if frm.size == 0:
        return 0.0
    row = np.asarray(row, dtype=np.int64)
    lab = _span_sectors(row[frm] * 4, row[frm + 1] * 4) * SECTOR
    last = _stops(p, length)
    tail = SECTOR * last.size + int(_span_sectors(row[last] * 4, row[last + 1] * 4).sum()) * SECTOR
    return (float((SECTOR + lab + SECTOR + 4).sum()) + tail) / frm.size


def metapath_index(paths: np.ndarray, row: np.ndarray, length: int) -> float:
    """Bytes per move of MetaPath walks answered from the label index: the
    wanted label's two CSR positions, one sorted neighbour and the path
    entry (no row pair; a walk that stops early is charged the positions
    read at its last vertex)."""
    frm, to, k, p = _moves(paths)
    if frm.size == 0:
        return 0.0
    last = _stops(p, length)
    return (frm.size * (SECTOR * 2 + 4) + SECTOR * last.size) / frm.size
