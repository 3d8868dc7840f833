"""The allocation-free dynamic-alias entry point.

trw_walk_dynamic_alias_noalloc serves callers that cannot allocate device
memory while they walk (a framework that owns every device byte through its
own pool, serving threads where an allocation would synchronise the device,
hosts with a fixed device-memory budget).  It keeps the dynamic-alias
kernel's per-warp tables in a fixed 16 MiB device array instead of memory
the library allocates.  These tests call it through the C ABI, twice in a
row, and require exactly the output of trw_walk (the existing entry point)
for the same walks: every walk is a pure function of (seed, walker, step),
so the two must agree bit for bit.  This file is collected last so that a
failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(N):
    L = N.load()
    f = L.trw_walk_dynamic_alias_noalloc
    P = ctypes.c_void_p
    f.argtypes = [P, ctypes.POINTER(N.WalkDesc), P, ctypes.c_int64, ctypes.c_int64, P, ctypes.c_int32, P, P, P, P]
    f.restype = ctypes.c_int
    return f


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("app_name", ["deepwalk", "node2vec", "metapath", "ppr", "genericwalk"])
def test_noalloc_matches_trw_walk_on_two_calls(app_name):
    from tests.gpu_util import need_gpu
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G

    g = G.make_graph("rmat", 1 << 12, 12, seed=77, labels=5)
    graph = E.Graph(g["row"], g["adj"], g["weight"], g["label"])
    try:
        L = 25
        # trw_walk runs dynamic-mode PPR and GenericWalk on the static alias
        # tables (walker-independent weights); this entry point always runs
        # the per-step dynamic kernel, so these two cases also check that
        # both forms give the same walks
        app = {"deepwalk": E.DeepWalk(L, mode="dynamic", sampler="alias"),
               "node2vec": E.Node2Vec(L, 2.0, 0.5, sampler="alias"),
               "metapath": E.MetaPath(L, [0, 1, 2, 3, 4], sampler="alias"),
               "ppr": E.PPR(0.25, mode="dynamic", sampler="alias"),
               "genericwalk": E.GenericWalk(L, mode="dynamic", sampler="alias")}[app_name]
        if app_name == "ppr":
            app.path_cap = L
        src = G.all_sources(g["row"], seed=3)[:3000].cuda()
        W = src.numel()
        ref = E.compute(graph, src, app, seed=5, id_base=11, count_visits=True)
        torch.cuda.synchronize()
        f = _entry(N)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for _ in range(2):
            paths = torch.full((W, L), -7, dtype=torch.int32, device="cuda")
            lengths = torch.full((W,), -7, dtype=torch.int32, device="cuda")
            counts = torch.zeros(graph.n, dtype=torch.int32, device="cuda")
            steps = torch.zeros(1, dtype=torch.int64, device="cuda")
            d = app.desc(5)
            N.check(f(graph.handle, ctypes.byref(d), _ptr(src), W, 11, _ptr(paths), L, _ptr(lengths), _ptr(counts),
                      _ptr(steps), stream))
            torch.cuda.synchronize()
            assert int(steps.item()) == ref.steps
            assert torch.equal(paths, ref.paths)
            assert torch.equal(lengths, ref.lengths)
            assert torch.equal(counts, ref.counts)
        assert graph.device_error() == 0
    finally:
        graph.close()


def test_noalloc_rejects_host_pointers_and_rows_above_its_limit():
    from tests.gpu_util import need_gpu
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N

    f = _entry(N)
    # star: vertex 0 has 70000 neighbours, above the 65535 limit of the fixed scratch
    leaves = 70000
    row = np.concatenate([[0, leaves], leaves + np.arange(1, leaves + 1)]).astype(np.int64)
    adj = np.concatenate([np.arange(1, leaves + 1), np.zeros(leaves)]).astype(np.int32)
    w = np.ones(adj.size)
    star = E.Graph(row, adj, w)
    try:
        src = torch.zeros(4, dtype=torch.int32, device="cuda")
        d = E.DeepWalk(5, mode="dynamic", sampler="alias").desc(1)
        rc = f(star.handle, ctypes.byref(d), _ptr(src), 4, 0, None, 0, None, None, None, None)
        assert rc == -7  # TRW_ERR_CAPACITY
        assert b"65535" in N.load().trw_last_error()
    finally:
        star.close()
    small = E.Graph(np.array([0, 1, 2], dtype=np.int64), np.array([1, 0], dtype=np.int32), np.ones(2))
    try:
        host_src = np.zeros(2, dtype=np.int32)
        d = E.DeepWalk(5, mode="dynamic", sampler="alias").desc(1)
        rc = f(small.handle, ctypes.byref(d), host_src.ctypes.data, 2, 0, None, 0, None, None, None, None)
        assert rc == -1  # TRW_ERR_INVALID: staging a host buffer would allocate
    finally:
        small.close()


def test_noalloc_node2vec_before_edge_set():
    """The first Node2Vec walk on a graph builds its edge set; the
    allocation-free entry point never does, so called first it runs the
    binary-search neighbour test.  Both forms must give the same walks."""
    from tests.gpu_util import need_gpu
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G

    g = G.make_graph("rmat", 1 << 12, 12, seed=78)
    graph = E.Graph(g["row"], g["adj"])
    try:
        L = 20
        app = E.Node2Vec(L, 2.0, 0.5, sampler="alias")
        src = G.all_sources(g["row"], seed=4)[:2000].cuda()
        W = src.numel()
        f = _entry(N)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        paths = torch.full((W, L), -7, dtype=torch.int32, device="cuda")
        lengths = torch.full((W,), -7, dtype=torch.int32, device="cuda")
        steps = torch.zeros(1, dtype=torch.int64, device="cuda")
        d = app.desc(6)
        rc = f(graph.handle, ctypes.byref(d), _ptr(src), W, 0, _ptr(paths), L, _ptr(lengths), None, _ptr(steps),
               stream)
        assert rc == 0, N.load().trw_last_error()
        ref = E.compute(graph, src, app, seed=6)  # builds the edge set
        torch.cuda.synchronize()
        assert torch.equal(paths, ref.paths) and torch.equal(lengths, ref.lengths)
        assert int(steps.item()) == ref.steps
    finally:
        graph.close()


def test_noalloc_is_profiled_and_holds_the_graph_lock():
    """With profiling on, trw_profile_read reports this entry point's own walk
    (not an earlier trw_walk's), and calls from several host threads on one
    stream give the walks of serial calls (the entry point takes the graph's
    lock while another thread's trw_walk builds the edge set)."""
    import threading

    from tests.gpu_util import need_gpu
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G

    g = G.make_graph("rmat", 1 << 12, 12, seed=79)
    graph = E.Graph(g["row"], g["adj"], g["weight"])
    try:
        L = 30
        app = E.Node2Vec(L, 2.0, 0.5, sampler="alias")
        src = G.all_sources(g["row"], seed=5)[:2500].cuda()
        W = src.numel()
        f = _entry(N)
        stream = torch.cuda.current_stream()
        sp = ctypes.c_void_p(stream.cuda_stream)
        # a short trw_walk first, so a stale reading would show its duration
        E.compute(graph, src[:64], E.DeepWalk(3, mode="dynamic", sampler="its"), seed=1)
        torch.cuda.synchronize()
        graph.profile(True)
        E.compute(graph, src[:64], E.DeepWalk(3, mode="dynamic", sampler="its"), seed=1)
        short_ms, _ = graph.last_timings()
        paths = torch.full((W, L), -7, dtype=torch.int32, device="cuda")
        lengths = torch.full((W,), -7, dtype=torch.int32, device="cuda")
        d = app.desc(8)
        N.check(f(graph.handle, ctypes.byref(d), _ptr(src), W, 0, _ptr(paths), L, _ptr(lengths), None, None, sp))
        walk_ms, post_ms = graph.last_timings()
        graph.profile(False)
        assert walk_ms > 0.0 and post_ms == 0.0
        assert walk_ms != short_ms
        # one thread builds the edge set through trw_walk while another calls the entry point
        out = {}

        def via_trw_walk():
            with torch.cuda.stream(stream):
                out["ref"] = E.compute(graph, src, app, seed=9)

        paths2 = torch.full((W, L), -7, dtype=torch.int32, device="cuda")
        lengths2 = torch.full((W,), -7, dtype=torch.int32, device="cuda")
        t = threading.Thread(target=via_trw_walk)
        t.start()
        d9 = app.desc(9)
        rc = f(graph.handle, ctypes.byref(d9), _ptr(src), W, 0, _ptr(paths2), L, _ptr(lengths2), None, None, sp)
        t.join()
        assert rc == 0, N.load().trw_last_error()
        torch.cuda.synchronize()
        assert torch.equal(paths2, out["ref"].paths) and torch.equal(lengths2, out["ref"].lengths)
        assert graph.device_error() == 0
    finally:
        graph.close()
