"""Seeded synthetic graph generators producing the reference's CSR layout.

The reference's edge-list converter (util/graph/graph.cpp:463-519, used by
toolset/edgelist_to_csr.cpp) makes every input undirected: it sorts the
(min, max) endpoint pairs, drops duplicates and self loops, and stores both
directions, so every neighbour list is sorted ascending (the property that
Graph::is_neighbor, graph.h:180-199, relies on).  ``to_csr`` builds the same
CSR from any edge list.  Weights follow the reference's AssignWeight tool in
shape (uniform per directed entry, toolset/assign_weight.cpp:34-35) but on
(0, 1] as the workloads here specify; labels follow AssignEdgeLabel
(toolset/assign_edge_label.cpp:32-33), uniform on [0, k).

All functions take a ``device`` so the same code builds small graphs on the
CPU for tests and the large workloads directly in HBM.  Each is deterministic
for a given (seed, device).
"""
from __future__ import annotations

import math

import torch


def _gen(seed: int, device) -> torch.Generator:
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    return g


def rmat_edges(scale: int, num_edges: int, a: float, b: float, c: float, seed: int,
               device="cpu", chunk: int = 1 << 24):
    """R-MAT (Chakrabarti, Zhan, Faloutsos 2004): each edge picks one of four
    quadrants per level with probabilities (a, b, c, 1-a-b-c)."""
    g = _gen(seed, device)
    srcs, dsts = [], []
    for start in range(0, num_edges, chunk):
        m = min(chunk, num_edges - start)
        src = torch.zeros(m, dtype=torch.int64, device=device)
        dst = torch.zeros(m, dtype=torch.int64, device=device)
        for level in range(scale):
            r = torch.rand(m, generator=g, device=device, dtype=torch.float64)
            bit = 1 << (scale - 1 - level)
            # quadrant 0: [0,a) -> (0,0); 1: [a,a+b) -> (0,1); 2: [a+b,a+b+c) -> (1,0); 3 -> (1,1)
            down = r >= (a + b)
            right = ((r >= a) & (r < a + b)) | (r >= a + b + c)
            src += down.to(torch.int64) * bit
            dst += right.to(torch.int64) * bit
            del r, down, right
        srcs.append(src)
        dsts.append(dst)
    return torch.cat(srcs), torch.cat(dsts)


def chung_lu_edges(n: int, avg_degree: float, gamma: float, seed: int, device="cpu"):
    """Chung-Lu power-law graph: expected degree of vertex i proportional to
    (i + 1)^(-1/(gamma-1)); n*avg_degree/2 endpoint pairs drawn independently
    in proportion to the expected degrees."""
    g = _gen(seed, device)
    i = torch.arange(n, dtype=torch.float64, device=device)
    w = (i + 1.0).pow(-1.0 / (gamma - 1.0))
    w = w * (avg_degree * n / w.sum())
    m = int(n * avg_degree / 2)
    cdf = torch.cumsum(w, 0)
    cdf = cdf / cdf[-1]
    u = torch.rand(m, generator=g, device=device, dtype=torch.float64)
    v = torch.rand(m, generator=g, device=device, dtype=torch.float64)
    src = torch.searchsorted(cdf, u).clamp_(max=n - 1)
    dst = torch.searchsorted(cdf, v).clamp_(max=n - 1)
    # scramble ids so that degree does not follow vertex id
    perm = torch.randperm(n, generator=g, device=device)
    return perm[src], perm[dst]


def erdos_renyi_edges(n: int, avg_degree: float, seed: int, device="cpu"):
    g = _gen(seed, device)
    m = int(n * avg_degree / 2)
    src = torch.randint(0, n, (m,), generator=g, device=device)
    dst = torch.randint(0, n, (m,), generator=g, device=device)
    return src, dst


def to_csr(n: int, src: torch.Tensor, dst: torch.Tensor):
    """Undirected, deduplicated, self-loop-free CSR with sorted neighbour lists
    (graph.cpp:463-519).  Returns (row int64[n+1], adj int32[e])."""
    keep = src != dst
    src, dst = src[keep], dst[keep]
    lo = torch.minimum(src, dst)
    hi = torch.maximum(src, dst)
    del src, dst, keep
    key = torch.unique(lo * n + hi)
    del lo, hi
    u = key // n
    v = key % n
    del key
    a = torch.cat([u, v])
    bb = torch.cat([v, u])
    del u, v
    key = torch.sort(a * n + bb).values
    del a, bb
    adj = (key % n).to(torch.int32)
    deg = torch.bincount(key // n, minlength=n)
    del key
    row = torch.zeros(n + 1, dtype=torch.int64, device=adj.device)
    torch.cumsum(deg, 0, out=row[1:])
    return row, adj


def uniform_weights(e: int, seed: int, device="cpu"):
    """Doubles uniform on (0, 1]: 1 - U[0, 1)."""
    g = _gen(seed, device)
    return 1.0 - torch.rand(e, generator=g, device=device, dtype=torch.float64)


def uniform_labels(e: int, k: int, seed: int, device="cpu"):
    g = _gen(seed, device)
    return torch.randint(0, k, (e,), generator=g, device=device, dtype=torch.int32)


def random_sources(row: torch.Tensor, count: int, seed: int):
    """``count`` sources drawn uniformly among non-isolated vertices (the
    shape of generate_random_source, walker_generator.cpp:27-40)."""
    g = _gen(seed, row.device)
    deg = row[1:] - row[:-1]
    nz = torch.nonzero(deg > 0).flatten()
    idx = torch.randint(0, nz.numel(), (count,), generator=g, device=row.device)
    return nz[idx].to(torch.int32)


def all_sources(row: torch.Tensor, seed: int | None = 0):
    """One walker per non-isolated vertex (generate_all_source,
    walker_generator.cpp:9-25), shuffled with a seeded permutation."""
    deg = row[1:] - row[:-1]
    nz = torch.nonzero(deg > 0).flatten().to(torch.int32)
    if seed is None:
        return nz
    g = _gen(seed, row.device)
    return nz[torch.randperm(nz.numel(), generator=g, device=row.device)]


def make_graph(kind: str, n: int, avg_degree: float, seed: int, device="cpu",
               weights: bool = True, labels: int = 0, **kw):
    """Convenience: generate edges, CSR, weights (0,1] and labels in [0, labels)."""
    if kind == "rmat":
        scale = int(math.log2(n))
        assert 1 << scale == n, "R-MAT needs a power-of-two vertex count"
        a, b, c = kw.get("a", 0.57), kw.get("b", 0.19), kw.get("c", 0.19)
        src, dst = rmat_edges(scale, int(n * avg_degree / 2), a, b, c, seed, device)
    elif kind == "chunglu":
        src, dst = chung_lu_edges(n, avg_degree, kw.get("gamma", 2.1), seed, device)
    elif kind == "er":
        src, dst = erdos_renyi_edges(n, avg_degree, seed, device)
    else:
        raise ValueError(kind)
    row, adj = to_csr(n, src, dst)
    e = adj.numel()
    out = {"n": n, "row": row, "adj": adj}
    out["weight"] = uniform_weights(e, seed + 1, device) if weights else None
    out["label"] = uniform_labels(e, labels, seed + 2, device) if labels else None
    return out
