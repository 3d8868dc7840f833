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


def philox_word(seed: int, walker: np.ndarray, step: np.ndarray, block: int, word: int) -> np.ndarray:
    """Word `word` of Philox4x32-10 (Salmon et al., SC'11) with key = seed and
    counter = (block, step, walker lo, walker hi): the engine's draw stream,
    vectorised over walkers and steps."""
    m = np.uint64(0xFFFFFFFF)
    walker = np.asarray(walker, dtype=np.uint64)
    c0 = np.full(walker.shape, block, dtype=np.uint64)
    c1 = np.asarray(step, dtype=np.uint64) & m
    c2 = walker & m
    c3 = walker >> np.uint64(32)
    k0, k1 = np.uint64(seed & 0xFFFFFFFF), np.uint64((seed >> 32) & 0xFFFFFFFF)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(0x9E3779B9)) & m
            k1 = (k1 + np.uint64(0xBB67AE85)) & m
        p0 = np.uint64(0xD2511F53) * c0
        p1 = np.uint64(0xCD9E8D57) * c2
        c0, c1, c2, c3 = ((p1 >> np.uint64(32)) ^ c1 ^ k0) & m, p1 & m, ((p0 >> np.uint64(32)) ^ c3 ^ k1) & m, p0 & m
    return (c0, c1, c2, c3)[word].astype(np.uint32)


def accept_threshold(max_weight: float, w: float) -> int:
    """Largest u in [0, 2^32) with (u * 2^-32) * max_weight <= w (the
    engine's integer form of the max-weight rejection test)."""
    lo, hi = 0, 0xFFFFFFFF
    while lo < hi:
        mid = lo + (hi - lo + 1) // 2
        if (mid * (1.0 / 4294967296.0)) * max_weight <= w:
            lo = mid
        else:
            hi = mid - 1
    return lo


def node2vec(paths: np.ndarray, length: int, seed=None, id_base: int = 0, p: float = 2.0, q: float = 0.5,
             fat: bool = False) -> float:
    """Bytes per move of Node2Vec walks with the edge-set neighbour test
    (walks that stop early are charged the row pair of their last vertex).
    With the walks' seed, a move is charged the probe only when the engine
    makes one: its first trial's acceptance draw lies above the lower of the
    common-neighbour and other-vertex thresholds (below it the move is
    accepted whatever the probe would say; a move accepted at a later trial
    is charged as if it had probed).  ``fat``: the adjacency entries carry
    the neighbours' row pairs, so a move reads its entry's sector and no row
    pair; only a walker's source row pair is read (at its admission)."""
    frm, to, k, pth = _moves(paths)
    if frm.size == 0:
        return 0.0
    # previous vertex of each move: path entry k-2 (none for the first move)
    prev = np.full(pth[:, :-1].shape, -1, dtype=np.int64)
    prev[:, 1:] = pth[:, :-2]
    valid = (pth[:, :-1] >= 0) & (pth[:, 1:] >= 0)
    prev = prev[valid]
    probe = (k >= 2) & (to != prev)
    if seed is not None:
        walker = np.broadcast_to(np.arange(pth.shape[0], dtype=np.int64)[:, None] + id_base, valid.shape)[valid]
        u = philox_word(int(seed), walker, k, 0, 1)  # trial 0: words 0 (position) and 1 (acceptance)
        mx = max(1.0, 1.0 / q, 1.0 / p)
        lo = min(accept_threshold(mx, 1.0), accept_threshold(mx, 1.0 / q))
        probe &= u > np.uint32(lo)
    if fat:
        total = frm.size * (SECTOR + 4) + int((k == 1).sum()) * SECTOR + int(probe.sum()) * SECTOR
    else:
        total = frm.size * (SECTOR + SECTOR + 4) + int(probe.sum()) * SECTOR + _stops(pth, length).size * SECTOR
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


def metapath_index(paths: np.ndarray, row: np.ndarray, length: int, fat: bool = False) -> float:
    """Bytes per move of MetaPath walks answered from the label index: the
    wanted label's two CSR positions, one sorted neighbour and the path
    entry (no row pair; a walk that stops early is charged the positions
    read at its last vertex).  ``fat``: the index entries carry the next
    step's positions, so a move reads its entry's sector and the path entry;
    only a walker's source positions are read (at its admission)."""
    frm, to, k, p = _moves(paths)
    if frm.size == 0:
        return 0.0
    if fat:
        walkers = int((np.asarray(p)[:, 0] >= 0).sum())
        return (frm.size * (SECTOR + 4) + SECTOR * walkers) / frm.size
    last = _stops(p, length)
    return (frm.size * (SECTOR * 2 + 4) + SECTOR * last.size) / frm.size


def sector_reuse(paths: np.ndarray, row: np.ndarray, adj: np.ndarray, cache_bytes=(227 << 10, 129 << 20)):
    """How much an ideal cache of the hottest 32-byte sectors could serve of
    the walks' random reads: for each cache size, the fraction of row-pair
    reads and of adjacency reads that fall in the most-read sectors of the
    whole sample (chosen with hindsight, so an upper bound for any staging of
    rows in shared memory or L2).  A move from u to v reads u's row pair
    (8-byte pairs) and the adjacency entry holding v in u's sorted row."""
    frm, to, _, _ = _moves(paths)
    row = np.asarray(row, dtype=np.int64)
    adj = np.asarray(adj)
    out = {"moves": int(frm.size)}
    if frm.size == 0:
        return out
    # position of `to` in frm's sorted row, searched row by row
    order = np.argsort(frm, kind="stable")
    f, t = frm[order], to[order]
    pos = np.empty(f.size, dtype=np.int64)
    starts = np.flatnonzero(np.r_[True, f[1:] != f[:-1]])
    ends = np.r_[starts[1:], f.size]
    for a, b in zip(starts, ends):
        u = f[a]
        lo, hi = row[u], row[u + 1]
        pos[a:b] = lo + np.searchsorted(adj[lo:hi], t[a:b])
    for name, sec in (("row_pair", f * 8 // SECTOR), ("adjacency", pos * 4 // SECTOR)):
        _, cnt = np.unique(sec, return_counts=True)
        cnt = np.sort(cnt)[::-1]
        cum = np.cumsum(cnt)
        out[name + "_distinct_sectors"] = int(cnt.size)
        for cb in cache_bytes:
            k = min(cnt.size, cb // SECTOR)
            out["%s_hit_%dKB" % (name, cb >> 10)] = float(cum[k - 1] / cum[-1]) if k > 0 else 0.0
    return out


def top_degree_share(paths: np.ndarray, row: np.ndarray, ks=(1024, 4096, 8192, 65536)):
    """Fraction of the moves that start at one of the k highest-degree
    vertices (their row pairs are what a shared-memory table of hub rows
    keyed by vertex could serve), for each k."""
    frm, _, _, _ = _moves(paths)
    deg = np.diff(np.asarray(row, dtype=np.int64))
    rank = np.empty(deg.size, dtype=np.int64)
    rank[np.argsort(-deg, kind="stable")] = np.arange(deg.size)
    r = rank[frm]
    return {int(k): float((r < k).mean()) if frm.size else 0.0 for k in ks}
