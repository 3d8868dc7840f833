"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, ``__graft_entry__.smoke()`` and the cpu_baseline/reference
legs of bench.py.  The product library never imports this module.

Also runs the reference-harness binaries (oracle/_ref/ref_<app>, built from
the reference sources where that tree exists) to pin the restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_APPS = ["deepwalk", "ppr", "node2vec", "metapath", "genericwalk"]

APPS = {"deepwalk": 0, "ppr": 1, "node2vec": 2, "metapath": 3, "genericwalk": 4}
MODES = {"uniform": 0, "static": 1, "dynamic": 2}
SAMPLERS = {"uniform": 0, "its": 1, "alias": 2, "rejection": 3, "maxweight_rejection": 4}

ALIAS_DTYPE = np.dtype([("prob", "<f8"), ("first", "<i4"), ("second", "<i4")])


class _Graph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("e", ctypes.c_int64),
                ("row", ctypes.c_void_p), ("adj", ctypes.c_void_p),
                ("weight", ctypes.c_void_p), ("label", ctypes.c_void_p),
                ("alias", ctypes.c_void_p), ("prefix", ctypes.c_void_p),
                ("rej_weight", ctypes.c_void_p), ("rej_max", ctypes.c_void_p)]


class _Desc(ctypes.Structure):
    _fields_ = [("app", ctypes.c_int32), ("mode", ctypes.c_int32), ("sampler", ctypes.c_int32),
                ("length", ctypes.c_int32), ("p", ctypes.c_double), ("q", ctypes.c_double),
                ("tp", ctypes.c_double), ("schema", ctypes.c_void_p), ("schema_len", ctypes.c_int32),
                ("seed", ctypes.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from oracle import build_oracle
            build_oracle.build(with_ref=False)
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.oracle_philox4x32_10.argtypes = [P, P, P]
        L.oracle_draw_u32.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        L.oracle_draw_u32.restype = ctypes.c_uint32
        for fn in ("oracle_build_alias", "oracle_build_prefix"):
            getattr(L, fn).argtypes = [P, ctypes.c_int, P]
        L.oracle_build_rejection.argtypes = [P, ctypes.c_int, P, P]
        L.oracle_walk.argtypes = [P, P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, P,
                                  ctypes.c_int32, P, P, P, ctypes.c_int32]
        L.oracle_walk_interleaved.argtypes = [P, P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, P,
                                              ctypes.c_int32, P, P, P, ctypes.c_int32, ctypes.c_int32]
        L.oracle_set_neighbor_accounting.argtypes = [ctypes.c_int32]
        L.oracle_set_neighbor_accounting.restype = None
        L.oracle_count_bytes.argtypes = [P, P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_int32, ctypes.c_int32, P, P, ctypes.c_int32]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def as_np(x, dtype):
    if x is None:
        return None
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


class Graph:
    """Host CSR (+ optional static tables) in the layout of graph.h:51-83."""

    def __init__(self, row, adj, weight=None, label=None):
        self.row = as_np(row, np.int64)
        self.adj = as_np(adj, np.int32)
        self.weight = as_np(weight, np.float64)
        self.label = as_np(label, np.int32)
        self.n = self.row.size - 1
        self.e = self.adj.size
        self.alias = self.prefix = self.rej_weight = self.rej_max = None

    def struct(self):
        return _Graph(self.n, self.e, _ptr(self.row), _ptr(self.adj), _ptr(self.weight), _ptr(self.label),
                      _ptr(self.alias), _ptr(self.prefix), _ptr(self.rej_weight), _ptr(self.rej_max))

    def build_tables(self, sampler, weight_kind=0):
        g = self.struct()
        if sampler == "alias":
            self.alias = np.zeros(self.e, dtype=ALIAS_DTYPE)
            rc = lib().oracle_build_alias(ctypes.byref(g), weight_kind, _ptr(self.alias))
        elif sampler == "its":
            self.prefix = np.zeros(self.e, dtype=np.float64)
            rc = lib().oracle_build_prefix(ctypes.byref(g), weight_kind, _ptr(self.prefix))
        elif sampler == "rejection":
            self.rej_weight = np.zeros(self.e, dtype=np.float64)
            self.rej_max = np.zeros(self.n, dtype=np.float64)
            rc = lib().oracle_build_rejection(ctypes.byref(g), weight_kind, _ptr(self.rej_weight),
                                              _ptr(self.rej_max))
        else:
            raise ValueError(sampler)
        if rc:
            raise RuntimeError("oracle table build failed: %d" % rc)


def make_desc(app, mode, sampler, length=80, p=1.0, q=1.0, tp=0.2, schema=None, seed=1):
    schema_arr = as_np(schema if schema is not None else [0], np.int32)
    d = _Desc(APPS[app], MODES[mode], SAMPLERS[sampler], int(length), float(p), float(q), float(tp),
              schema_arr.ctypes.data, int(schema_arr.size if schema is not None else 0), int(seed))
    d._keep = schema_arr
    return d


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out


def draw_u32(seed, walker, step, d):
    return lib().oracle_draw_u32(seed, walker, step, d)


def walk(graph: Graph, desc, sources, per_query=0, id_base=0, path_cap=0, want_lengths=True,
         want_counts=False, num_queries=None, threads=0, interleaved=False, ring=64, out_counts=None):
    """Runs the oracle walks; returns dict(paths, lengths, counts, steps).
    ``out_counts`` (int32, C-contiguous, num_queries x n) receives the visit
    counts added in place instead of a fresh array."""
    src = as_np(sources, np.int32)
    W = src.size * per_query if per_query > 0 else src.size
    paths = np.full((W, path_cap), -1, dtype=np.int32) if path_cap > 0 else None
    lengths = np.zeros(W, dtype=np.int32) if want_lengths else None
    nq = (src.size if per_query > 0 else 1) if num_queries is None else num_queries
    if out_counts is not None:
        assert out_counts.dtype == np.int32 and out_counts.flags.c_contiguous and out_counts.size >= nq * graph.n
        counts = out_counts
    else:
        counts = np.zeros((nq, graph.n), dtype=np.int32) if want_counts else None
    steps = ctypes.c_uint64(0)
    g = graph.struct()
    if interleaved:
        rc = lib().oracle_walk_interleaved(ctypes.byref(g), ctypes.byref(desc), _ptr(src), W, per_query,
                                           id_base, _ptr(paths), path_cap, _ptr(lengths), _ptr(counts),
                                           ctypes.byref(steps), threads, ring)
    else:
        rc = lib().oracle_walk(ctypes.byref(g), ctypes.byref(desc), _ptr(src), W, per_query, id_base,
                               _ptr(paths), path_cap, _ptr(lengths), _ptr(counts), ctypes.byref(steps),
                               threads)
    if rc:
        raise RuntimeError("oracle walk failed: %d" % rc)
    return {"paths": paths, "lengths": lengths, "counts": counts, "steps": steps.value}


def count_bytes(graph: Graph, desc, sources, per_query=0, id_base=0, record_paths=True,
                count_visits=False, threads=0, neighbor_probe=False, label_index=False):
    """Algorithmic bytes (32-byte sectors per independent access) and steps
    of the walks.  ``neighbor_probe`` charges Node2Vec's neighbour test as one
    hash probe (the GPU engine on a symmetric graph) instead of the
    reference's binary search; ``label_index`` charges MetaPath's label scan
    as one read of a label index's offsets."""
    lib().oracle_set_neighbor_accounting((1 if neighbor_probe else 0) | (2 if label_index else 0))
    src = as_np(sources, np.int32)
    W = src.size * per_query if per_query > 0 else src.size
    nbytes = ctypes.c_uint64(0)
    steps = ctypes.c_uint64(0)
    g = graph.struct()
    rc = lib().oracle_count_bytes(ctypes.byref(g), ctypes.byref(desc), _ptr(src), W, per_query, id_base,
                                  int(record_paths), int(count_visits), ctypes.byref(nbytes),
                                  ctypes.byref(steps), threads)
    if rc:
        raise RuntimeError("oracle count failed: %d" % rc)
    return nbytes.value, steps.value


def have_reference_harness():
    return all(os.path.exists(os.path.join(REF_DIR, "ref_" + a)) for a in REF_APPS)


def run_reference(graph: Graph, app, mode, sampler, sources, length=80, path_cap=80, seed=1, id_base=0,
                  p=1.0, q=1.0, tp=0.2, schema=None):
    """Runs the reference's own samplers (oracle/_ref harness) on one graph."""
    exe = os.path.join(REF_DIR, "ref_" + app)
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    with tempfile.TemporaryDirectory() as d:
        graph.row.tofile(os.path.join(d, "row.bin"))
        graph.adj.tofile(os.path.join(d, "adj.bin"))
        as_np(sources, np.int32).tofile(os.path.join(d, "sources.bin"))
        if graph.weight is not None:
            graph.weight.tofile(os.path.join(d, "weight.bin"))
        if graph.label is not None:
            graph.label.tofile(os.path.join(d, "label.bin"))
        args = [exe, d, str(MODES[mode]), str(SAMPLERS[sampler]), str(length), str(path_cap), str(seed),
                str(id_base), repr(float(p)), repr(float(q)), repr(float(tp))]
        args += [str(int(s)) for s in (schema or [])]
        subprocess.run(args, check=True)
        W = as_np(sources, np.int32).size
        out = {
            "paths": np.fromfile(os.path.join(d, "paths.bin"), dtype=np.int32).reshape(W, max(path_cap, 1)),
            "lengths": np.fromfile(os.path.join(d, "lengths.bin"), dtype=np.int32),
            "counts": np.fromfile(os.path.join(d, "counts.bin"), dtype=np.int32),
            "steps": int(open(os.path.join(d, "steps.txt")).read()),
        }
        for name, dt in (("alias", ALIAS_DTYPE), ("prefix", np.float64), ("rejw", np.float64),
                         ("rejmax", np.float64)):
            f = os.path.join(d, name + ".bin")
            if os.path.exists(f):
                out[name] = np.fromfile(f, dtype=dt)
        return out
