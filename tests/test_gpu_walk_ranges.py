"""trw_walk into host buffers for a large batch runs as walker ranges whose
copies overlap the next range's walk; the paths, lengths, visit counts and
step count equal those of the same walks into device buffers."""
import ctypes

import numpy as np
import pytest

from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("app_name,pinned", [("deepwalk", False), ("node2vec", True), ("metapath", True)])
def test_host_ranges_equal_device_walk(app_name, pinned):
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 12, 12, seed=81, labels=5)
    graph = E.Graph(g["row"], g["adj"], g["weight"], g["label"])
    try:
        L = 10
        app = {"deepwalk": E.DeepWalk(L), "node2vec": E.Node2Vec(L, 2.0, 0.5),
               "metapath": E.MetaPath(L, [0, 1, 2, 3, 4])}[app_name]
        base = G.all_sources(g["row"], seed=2).to(torch.int32)
        W = 1_400_000  # > 4 walkers per lane of 152 SMs: several ranges
        src = base.repeat((W + base.numel() - 1) // base.numel())[:W].contiguous()
        dev = E.compute(graph, src.cuda(), app, seed=8, id_base=5, count_visits=True)
        torch.cuda.synchronize()

        def host(shape, dtype):
            t = torch.zeros(shape, dtype=dtype)
            return t.pin_memory() if pinned else t
        paths, lengths = host((W, L), torch.int32), host(W, torch.int32)
        counts, steps = host(graph.n, torch.int32), host(1, torch.int64)
        counts += 3  # trw_walk adds to the caller's counts
        hsrc = src.pin_memory() if pinned else src
        d = app.desc(8)
        rc = N.load().trw_walk(graph.handle, ctypes.byref(d), hsrc.data_ptr(), W, 5, paths.data_ptr(), L,
                               lengths.data_ptr(), counts.data_ptr(), steps.data_ptr(), 0, None)
        assert rc == 0, N.load().trw_last_error()
        assert int(steps[0]) == dev.steps
        assert torch.equal(paths, dev.paths.cpu())
        assert torch.equal(lengths, dev.lengths.cpu())
        assert torch.equal(counts - 3, dev.counts.cpu())
    finally:
        graph.close()


def test_host_ranges_errors_leave_graph_usable():
    """A ranged host-output walk that fails -- a bad descriptor before any
    range runs, an invalid source vertex inside one range -- returns its
    status after the queued ranges finish; the next call on the same graph
    gives the device-output walks exactly."""
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 12, 12, seed=83)
    graph = E.Graph(g["row"], g["adj"], g["weight"])
    L = N.load()
    try:
        app, Lw, W = E.DeepWalk(8), 8, 1_400_000
        base = G.all_sources(g["row"], seed=4).to(torch.int32)
        src = base.repeat((W + base.numel() - 1) // base.numel())[:W].contiguous().pin_memory()
        paths = torch.zeros((W, Lw), dtype=torch.int32).pin_memory()
        lengths = torch.zeros(W, dtype=torch.int32).pin_memory()

        def call(s, d):
            return L.trw_walk(graph.handle, ctypes.byref(d), s.data_ptr(), W, 0, paths.data_ptr(), Lw,
                              lengths.data_ptr(), None, None, 0, None)
        bad = app.desc(9)
        bad.app = 99
        assert call(src, bad) in (-1, -3)  # TRW_ERR_INVALID / TRW_ERR_UNSUPPORTED
        broken = src.clone().pin_memory()
        broken[W // 2 + 7] = graph.n + 5  # rejected at admission, no read outside the graph
        assert call(broken, app.desc(9)) == -6, L.trw_last_error()  # TRW_ERR_DEVICE
        assert call(src, app.desc(9)) == 0, L.trw_last_error()
        dev = E.compute(graph, src.cuda(), app, seed=9)
        torch.cuda.synchronize()
        assert torch.equal(paths, dev.paths.cpu())
        assert torch.equal(lengths, dev.lengths.cpu())
    finally:
        graph.close()


def test_sparse_host_ranges_capacity_retry():
    """A ranged sparse PPR batch into host buffers that are too small reports
    TRW_ERR_CAPACITY with offsets[Q] = the entries needed; the retry with that
    capacity gives the device-output batch entry for entry."""
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 13, 16, seed=21)
    Q, wpq = 61, 160_000  # several query ranges
    qs = G.random_sources(g["row"], Q, seed=9)
    graph = E.Graph(g["row"], g["adj"])
    L = N.load()
    try:
        dev = E.ppr_batch_sparse(graph, qs, wpq, tp=0.2, seed=41)
        need = int(dev.offsets[-1].item())
        src = qs.to(torch.int32).contiguous().pin_memory()
        off = torch.zeros(Q + 1, dtype=torch.int64).pin_memory()

        def call(cap):
            v = torch.zeros(max(cap, 1), dtype=torch.int32).pin_memory()
            c = torch.zeros(max(cap, 1), dtype=torch.int32).pin_memory()
            d = E.PPR(0.2).desc(41)
            rc = L.trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), src.data_ptr(), Q, wpq, off.data_ptr(),
                                        v.data_ptr(), c.data_ptr(), cap, None, 0, None)
            return rc, v, c
        rc, _, _ = call(need // 2)
        assert rc == -7, L.trw_last_error()  # TRW_ERR_CAPACITY
        assert int(off[-1]) == need
        rc, v, c = call(need)
        assert rc == 0, L.trw_last_error()
        assert torch.equal(off, dev.offsets.cpu())
        assert torch.equal(v[:need], dev.vertices[:need].cpu())
        assert torch.equal(c[:need], dev.counts[:need].cpu())
    finally:
        graph.close()
