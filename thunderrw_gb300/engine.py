"""Host-side mirror of ThunderRW's walk interface over libtrw_gpu.so.

Reference shape (random_walk/creeper.h:689, apps/*.cpp):

    Graph graph; graph.load_csr(dir);                  // util/graph/graph.cpp:45
    std::vector<WalkerMeta> walkers; generate_*(graph, walkers, ...);
    compute(graph, walkers, DeepWalk(l, &graph));      // mode/sampler from g_para

Here:

    g = Graph(row, adj, weight, label)                 # or Graph.load_csr(dir, ...)
    res = compute(g, sources, DeepWalk(80))            # app carries its g_para defaults
    res.paths, res.lengths, res.steps

Device memory and streams come from PyTorch (plumbing only); every walk and
table build runs in the CUDA library.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np
import torch

from . import _native as N


def _lib():
    return N.load()


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def _dev(x, dtype, device):
    if x is None:
        return None
    if not torch.is_tensor(x):
        x = torch.from_numpy(np.ascontiguousarray(np.asarray(x)))
    return x.to(device=device, dtype=dtype).contiguous()


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


# ---------------------------------------------------------------------------
# Apps: the five reference functors with their g_para defaults
# ---------------------------------------------------------------------------

@dataclass
class App:
    name: str
    mode: str
    sampler: str
    length: int = 80
    p: float = 1.0
    q: float = 1.0
    tp: float = 0.2
    schema: Optional[Sequence[int]] = None
    path_cap: Optional[int] = None

    def desc(self, seed: int, mode: Optional[str] = None, sampler: Optional[str] = None) -> N.WalkDesc:
        schema = np.ascontiguousarray(np.asarray(self.schema if self.schema is not None else [0], dtype=np.int32))
        d = N.WalkDesc(N.APPS[self.name], N.MODES[mode or self.mode], N.SAMPLERS[sampler or self.sampler],
                       int(self.length), float(self.p), float(self.q), float(self.tp),
                       schema.ctypes.data, int(len(self.schema)) if self.schema is not None else 0, int(seed))
        d._keep = schema
        return d

    def default_path_cap(self) -> int:
        # g_para.length_: l for the fixed-length apps, 1 for PPR (ppr.cpp:123)
        if self.path_cap is not None:
            return self.path_cap
        return 1 if self.name == "ppr" else self.length


def DeepWalk(l: int = 80, mode: str = "static", sampler: str = "alias") -> App:
    """deepwalk.cpp:7-30: Static + Alias, l = 80, weight = edge weight."""
    return App("deepwalk", mode, sampler, length=l)


def PPR(tp: float = 0.2, mode: str = "uniform", sampler: str = "uniform") -> App:
    """ppr.cpp:80-106: Uniform, stop with probability tp after every move."""
    return App("ppr", mode, sampler, length=1, tp=tp)


def Node2Vec(l: int = 80, p: float = 2.0, q: float = 0.5, mode: str = "dynamic",
             sampler: str = "maxweight_rejection") -> App:
    """node2vec.cpp:165-205: Dynamic + max-weight rejection; weights 1/p, 1, 1/q."""
    return App("node2vec", mode, sampler, length=l, p=p, q=q)


def MetaPath(l: int = 80, schema: Sequence[int] = (0, 1, 2, 3, 4), mode: str = "dynamic",
             sampler: str = "its") -> App:
    """metapath.cpp:7-39: Dynamic + ITS over the label filter."""
    return App("metapath", mode, sampler, length=l, schema=list(schema))


def GenericWalk(l: int = 80, mode: str = "static", sampler: str = "alias") -> App:
    """genericwalk.cpp:110-133."""
    return App("genericwalk", mode, sampler, length=l)


# ---------------------------------------------------------------------------
# Graph
# ---------------------------------------------------------------------------

ALIAS_DTYPE = np.dtype([("prob", "<f8"), ("first", "<i4"), ("second", "<i4")])


class Graph:
    """A CSR graph resident in HBM (the reference's Graph, graph.h:19-329)."""

    def __init__(self, row, adj, weight=None, label=None, check_sorted: bool = False, device=None):
        L = _lib()
        self.device = torch.device(device or "cuda")
        row = _dev(row, torch.int64, self.device)
        adj = _dev(adj, torch.int32, self.device)
        w = _dev(weight, torch.float64, self.device)
        lab = _dev(label, torch.int32, self.device)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            N.check(L.trw_graph_create(_ptr(row), _ptr(adj), _ptr(w), _ptr(lab), int(row.numel() - 1),
                                       int(adj.numel()), 1 if check_sorted else 0, ctypes.byref(h)))
        self._h = h
        n, e, md = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
        N.check(L.trw_graph_info(h, ctypes.byref(n), ctypes.byref(e), ctypes.byref(md)))
        self.n, self.e, self.max_degree_ = n.value, e.value, md.value
        self.has_weight = weight is not None
        self.has_label = label is not None

    @property
    def handle(self):
        return self._h

    def num_vertices(self) -> int:
        return self.n

    def num_edges(self) -> int:
        return self.e

    def max_degree(self) -> int:
        return self.max_degree_

    def build_tables(self, sampler: str, weights: str = "edge", stream=None):
        N.check(_lib().trw_tables_build(self._h, N.SAMPLERS[sampler], N.WEIGHTS[weights],
                                        ctypes.c_void_p(_stream_ptr(stream))))

    def download_table(self, sampler: str) -> np.ndarray:
        if sampler == "alias":
            out = np.zeros(self.e, dtype=ALIAS_DTYPE)
        elif sampler == "its":
            out = np.zeros(self.e, dtype=np.float64)
        elif sampler == "rejection":
            out = np.zeros(self.n, dtype=np.float64)
        else:
            raise ValueError(sampler)
        N.check(_lib().trw_tables_download(self._h, N.SAMPLERS[sampler], out.ctypes.data, out.nbytes))
        return out

    def upload_table(self, sampler: str, table, weights: str = "edge", stream=None):
        """Installs a precomputed table (trw_tables_upload): an AliasSlot
        array, ITS prefix sums or rejection maxima, e.g. read from the
        reference's b_edge_weight_*.bin files."""
        arr = np.ascontiguousarray(table)
        N.check(_lib().trw_tables_upload(self._h, N.SAMPLERS[sampler], N.WEIGHTS[weights], arr.ctypes.data,
                                         arr.nbytes, ctypes.c_void_p(_stream_ptr(stream))))

    def set_engine_shape(self, sampler: str, walkers_per_thread: int = 0, ctas_per_sm: int = 0):
        N.check(_lib().trw_set_engine_shape(self._h, N.SAMPLERS[sampler], walkers_per_thread, ctas_per_sm))

    def engine_shape(self, sampler: str):
        a, b = ctypes.c_int32(), ctypes.c_int32()
        N.check(_lib().trw_get_engine_shape(self._h, N.SAMPLERS[sampler], ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def profile(self, enable: bool = True):
        N.check(_lib().trw_profile_enable(self._h, 1 if enable else 0))

    def last_timings(self):
        """(walk kernel ms, post-processing ms) of the last walk call (profiling on)."""
        a, b = ctypes.c_float(), ctypes.c_float()
        N.check(_lib().trw_profile_read(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def indexes(self):
        """(edge set, label index) states: 0 not built yet, 1 built, -1 not
        applicable or no room (the walks then search, with the same results)."""
        a, b = ctypes.c_int32(), ctypes.c_int32()
        N.check(_lib().trw_graph_indexes(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def layout(self):
        """(fat adjacency, fat label index) states: 1 if the uniform and
        max-weight rejection walks read the 16-byte adjacency entries carrying
        each neighbour's row pair / if MetaPath walks with the last
        unique-label schema read label-index entries carrying the next step's
        block, -1 if not, 0 if no walk has decided it yet."""
        a, b = ctypes.c_int32(), ctypes.c_int32()
        N.check(_lib().trw_graph_layout(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def fat_adjacency(self) -> int:
        return self.layout()[0]

    def build_indexes(self, edge_set: bool = True, label_index: bool = True, stream=None):
        """Builds the Node2Vec edge set and / or the MetaPath label index now
        (e.g. before serving) instead of in the first walk that needs them;
        returns the states as indexes() does."""
        N.check(_lib().trw_graph_build_indexes(self._h, 1 if edge_set else 0, 1 if label_index else 0,
                                               ctypes.c_void_p(_stream_ptr(stream))))
        return self.indexes()

    def device_error(self) -> int:
        c = ctypes.c_int32()
        N.check(_lib().trw_device_error(self._h, ctypes.byref(c)))
        return c.value

    def close(self):
        if getattr(self, "_h", None):
            _lib().trw_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @classmethod
    def load_csr(cls, graph_dir: str, edge_weight: bool = False, edge_label: bool = False, **kw) -> "Graph":
        from . import formats
        d = formats.load_csr(graph_dir, edge_weight=edge_weight, edge_label=edge_label)
        return cls(d["row"], d["adj"], d.get("weight"), d.get("label"), **kw)


# ---------------------------------------------------------------------------
# Walks
# ---------------------------------------------------------------------------

@dataclass
class WalkResult:
    paths: Optional[torch.Tensor]
    lengths: Optional[torch.Tensor]
    counts: Optional[torch.Tensor]
    steps_dev: torch.Tensor = field(repr=False)

    @property
    def steps(self) -> int:
        return int(self.steps_dev.item())


def compute(graph: Graph, sources, app: App, mode: Optional[str] = None, sampler: Optional[str] = None,
            seed: int = 1, id_base: int = 0, record_paths: bool = True, path_cap: Optional[int] = None,
            count_visits: bool = False, engine: str = "persistent", stream=None) -> WalkResult:
    """compute<F>(graph, walkers, f) (creeper.h:689): walks one walker per entry
    of ``sources`` to completion.  Outputs are device tensors; the call is
    asynchronous on ``stream`` (``result.steps`` synchronises)."""
    dev = graph.device
    src = _dev(sources, torch.int32, dev)
    W = src.numel()
    cap = path_cap if path_cap is not None else app.default_path_cap()
    paths = torch.empty((W, cap), dtype=torch.int32, device=dev) if record_paths else None
    lengths = torch.empty(W, dtype=torch.int32, device=dev)
    counts = torch.zeros(graph.n, dtype=torch.int32, device=dev) if count_visits else None
    steps = torch.zeros(1, dtype=torch.int64, device=dev)
    d = app.desc(seed, mode, sampler)
    N.check(_lib().trw_walk(graph.handle, ctypes.byref(d), _ptr(src), W, int(id_base), _ptr(paths),
                            int(cap) if record_paths else 0, _ptr(lengths), _ptr(counts), _ptr(steps),
                            N.ENGINES[engine], ctypes.c_void_p(_stream_ptr(stream))))
    return WalkResult(paths, lengths, counts, steps)


def ppr_batch(graph: Graph, sources, walkers_per_query: int, tp: float = 0.2, seed: int = 1,
              counts: Optional[torch.Tensor] = None, zero_counts: bool = True, engine: str = "persistent",
              stream=None, mode: str = "uniform", sampler: str = "uniform"):
    """Batched PPR: len(sources) queries x walkers_per_query walkers in one
    launch; returns (counts[num_queries, n] int32 on the device, steps tensor).
    `mode` / `sampler` as the reference's -em / -sm (PPR's hook weighs every
    edge 1)."""
    dev = graph.device
    src = _dev(sources, torch.int32, dev)
    Q = src.numel()
    if counts is None:
        counts = torch.empty((Q, graph.n), dtype=torch.int32, device=dev)
        zero_counts = True
    steps = torch.zeros(1, dtype=torch.int64, device=dev)
    d = PPR(tp, mode, sampler).desc(seed)
    N.check(_lib().trw_ppr_batch(graph.handle, ctypes.byref(d), _ptr(src), Q, int(walkers_per_query), _ptr(counts),
                                 _ptr(steps), 1 if zero_counts else 0, N.ENGINES[engine],
                                 ctypes.c_void_p(_stream_ptr(stream))))
    return counts, steps


@dataclass
class SparseCounts:
    """Per-query visit counts in CSR form: query q's vertices are
    ``vertices[offsets[q]:offsets[q+1]]`` with ``counts`` alongside."""
    offsets: torch.Tensor
    vertices: torch.Tensor
    counts: torch.Tensor
    steps_dev: torch.Tensor = field(repr=False)

    @property
    def steps(self) -> int:
        return int(self.steps_dev.item())

    def dense(self, n: int) -> torch.Tensor:
        q = self.offsets.numel() - 1
        out = torch.zeros((q, n), dtype=torch.int32, device=self.vertices.device)
        total = int(self.offsets[-1].item())
        rows = torch.repeat_interleave(torch.arange(q, device=self.vertices.device),
                                       (self.offsets[1:] - self.offsets[:-1]))
        out[rows, self.vertices[:total].long()] = self.counts[:total]
        return out


def ppr_batch_sparse(graph: Graph, sources, walkers_per_query: int, tp: float = 0.2, seed: int = 1,
                     capacity: Optional[int] = None, engine: str = "persistent", stream=None,
                     out: Optional[SparseCounts] = None) -> SparseCounts:
    """Batched PPR with sparse per-query (vertex, count) output
    (trw_ppr_batch_sparse).  If the output does not fit ``capacity`` entries,
    the batch is rerun with the exact size (results are identical)."""
    dev = graph.device
    src = _dev(sources, torch.int32, dev)
    Q = src.numel()
    if out is None:
        if capacity is None:
            capacity = Q * min(graph.n, max(1, int(walkers_per_query * 3)))
        out = SparseCounts(torch.empty(Q + 1, dtype=torch.int64, device=dev),
                           torch.empty(max(1, capacity), dtype=torch.int32, device=dev),
                           torch.empty(max(1, capacity), dtype=torch.int32, device=dev),
                           torch.zeros(1, dtype=torch.int64, device=dev))
    cap = out.vertices.numel()
    d = PPR(tp).desc(seed)
    N.check(_lib().trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), _ptr(src), Q, int(walkers_per_query),
                                        _ptr(out.offsets), _ptr(out.vertices), _ptr(out.counts), cap,
                                        _ptr(out.steps_dev), N.ENGINES[engine], ctypes.c_void_p(_stream_ptr(stream))))
    total = int(out.offsets[-1].item())
    if total > cap:
        graph.device_error()  # clears the capacity flag of the first attempt
        out = SparseCounts(out.offsets, torch.empty(total, dtype=torch.int32, device=dev),
                           torch.empty(total, dtype=torch.int32, device=dev), out.steps_dev)
        return ppr_batch_sparse(graph, src, walkers_per_query, tp, seed, engine=engine, stream=stream, out=out)
    return out
