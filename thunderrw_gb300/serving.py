"""Python front end of the request loop in libtrw_gpu.so (trw_server_*).

The server keeps a graph and its sampling tables resident, admits requests
in arrival order whenever a stream slot is free and their device memory fits
the budget, and runs each admitted request on its own stream so requests that
arrive while others run overlap them on the device.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native as N
from .engine import App, Graph, PPR


class _Request(ctypes.Structure):
    _fields_ = [("desc", N.WalkDesc), ("sources", ctypes.c_void_p), ("num_walkers", ctypes.c_int64),
                ("id_base", ctypes.c_int64), ("path_cap", ctypes.c_int32), ("num_queries", ctypes.c_int64),
                ("walkers_per_query", ctypes.c_int64)]


class _Status(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("latency_ms", ctypes.c_double), ("queue_ms", ctypes.c_double),
                ("steps", ctypes.c_uint64), ("entries", ctypes.c_int64)]


class _Stats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("queued", ctypes.c_int64), ("running", ctypes.c_int64),
                ("hbm_in_use", ctypes.c_size_t), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("elapsed_s", ctypes.c_double), ("batches", ctypes.c_uint64)]


def _bind():
    L = N.load()
    if getattr(L, "_trw_server_bound", False):
        return L
    P = ctypes.c_void_p
    L.trw_server_start.argtypes = [P, ctypes.c_size_t, ctypes.c_int32, ctypes.POINTER(P)]
    L.trw_server_submit.argtypes = [P, ctypes.POINTER(_Request), ctypes.POINTER(ctypes.c_uint64)]
    L.trw_server_wait.argtypes = [P, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(_Status)]
    L.trw_server_result.argtypes = [P, ctypes.c_uint64, P, P, P, P, P, ctypes.c_int64]
    L.trw_server_release.argtypes = [P, ctypes.c_uint64]
    L.trw_server_stats.argtypes = [P, ctypes.POINTER(_Stats)]
    L.trw_server_stop.argtypes = [P]
    for f in ("trw_server_start", "trw_server_submit", "trw_server_wait", "trw_server_result", "trw_server_release",
              "trw_server_stats", "trw_server_stop"):
        getattr(L, f).restype = ctypes.c_int
    L._trw_server_bound = True
    return L


@dataclass
class RequestStatus:
    state: int
    latency_ms: float
    queue_ms: float
    steps: int
    entries: int


class Server:
    def __init__(self, graph: Graph, hbm_budget_bytes: int = 0, max_inflight: int = 8):
        self.L = _bind()
        self.graph = graph
        h = ctypes.c_void_p()
        N.check(self.L.trw_server_start(graph.handle, int(hbm_budget_bytes), int(max_inflight), ctypes.byref(h)))
        self._h = h
        self._keep = {}

    def submit_walk(self, app: App, sources, seed: int = 1, id_base: int = 0, path_cap: Optional[int] = None,
                    mode: Optional[str] = None, sampler: Optional[str] = None) -> int:
        src = np.ascontiguousarray(np.asarray(sources, dtype=np.int32))
        cap = app.default_path_cap() if path_cap is None else path_cap
        r = _Request(app.desc(seed, mode, sampler), src.ctypes.data, src.size, int(id_base), int(cap), 0, 0)
        t = ctypes.c_uint64()
        N.check(self.L.trw_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        self._keep[t.value] = ("walk", src.size, cap)
        return t.value

    def submit_ppr(self, sources, walkers_per_query: int, tp: float = 0.2, seed: int = 1) -> int:
        src = np.ascontiguousarray(np.asarray(sources, dtype=np.int32))
        r = _Request(PPR(tp).desc(seed), src.ctypes.data, 0, 0, 0, src.size, int(walkers_per_query))
        t = ctypes.c_uint64()
        N.check(self.L.trw_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        self._keep[t.value] = ("ppr", src.size, 0)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> RequestStatus:
        st = _Status()
        N.check(self.L.trw_server_wait(self._h, ticket, int(timeout_ms), ctypes.byref(st)))
        return RequestStatus(st.state, st.latency_ms, st.queue_ms, st.steps, st.entries)

    def result(self, ticket: int):
        kind, n, cap = self._keep[ticket]
        st = self.wait(ticket)
        if kind == "walk":
            lengths = np.zeros(n, dtype=np.int32)
            paths = np.zeros((n, cap), dtype=np.int32) if cap > 0 else None
            N.check(self.L.trw_server_result(self._h, ticket, None if paths is None else paths.ctypes.data,
                                             lengths.ctypes.data, None, None, None, 0))
            return {"paths": paths, "lengths": lengths, "steps": st.steps}
        offsets = np.zeros(n + 1, dtype=np.int64)
        v = np.zeros(max(1, st.entries), dtype=np.int32)
        c = np.zeros(max(1, st.entries), dtype=np.int32)
        N.check(self.L.trw_server_result(self._h, ticket, None, None, offsets.ctypes.data, v.ctypes.data,
                                         c.ctypes.data, v.size))
        return {"offsets": offsets, "vertices": v[:st.entries], "counts": c[:st.entries], "steps": st.steps}

    def release(self, ticket: int):
        N.check(self.L.trw_server_release(self._h, ticket))
        self._keep.pop(ticket, None)

    def stats(self) -> dict:
        s = _Stats()
        N.check(self.L.trw_server_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _Stats._fields_}

    def stop(self):
        if getattr(self, "_h", None):
            self.L.trw_server_stop(self._h)
            self._h = None

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass
