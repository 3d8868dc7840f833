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
