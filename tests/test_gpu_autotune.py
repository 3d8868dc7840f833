"""The launch-shape autotuner: it times every candidate, sets the fastest on
the graph, and walks stay identical under the tuned shape."""
import numpy as np
import pytest

from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu


def test_tune_sets_fastest_shape_and_keeps_results():
    torch, E = need_gpu()
    from thunderrw_gb300 import autotune
    from thunderrw_gb300 import generators as G
    g = G.make_graph("chunglu", 1 << 12, 10, seed=4)
    graph = E.Graph(g["row"], g["adj"], g["weight"])
    try:
        src = G.all_sources(g["row"], seed=0)
        app = E.DeepWalk(12)
        before = E.compute(graph, src, app, seed=5)
        res = autotune.tune(graph, app, src, rings=(1, 4), ctas=(0, 2), repeats=1)
        assert set(res.timings) == {(0, 0), (1, 0), (1, 2), (4, 0), (4, 2), (-1, 0)}
        fastest = min(res.timings, key=res.timings.get)
        # the automatic shape stays unless beaten by more than 3 %
        assert res.best in (fastest, (0, 0))
        assert res.timings[res.best] <= res.timings[fastest] * 1.03 + 1e-9
        assert graph.engine_shape("alias") == res.best
        after = E.compute(graph, src, app, seed=5)
        assert torch.equal(before.paths, after.paths) and before.steps == after.steps
        # sparse PPR tunes the uniform slot
        r2 = autotune.tune(graph, E.PPR(0.2), src[:8], walkers_per_query=2000, rings=(1, 2), ctas=(0,), repeats=1)
        assert r2.sampler == "uniform" and set(r2.timings) == {(0, 0), (1, 0), (2, 0), (-1, 0)}
        # Node2Vec's dynamic ITS (walker-dependent weights, one warp per walker step): CTAs only
        r3 = autotune.tune(graph, E.Node2Vec(6, 2.0, 0.5, sampler="its"), src, ctas=(0, 1), repeats=1)
        assert r3.sampler == "its" and set(r3.timings) == {(0, 0), (0, 1)}
        # DeepWalk's dynamic ITS runs on the static tables: rings are tuned too
        r4 = autotune.tune(graph, E.DeepWalk(6, mode="dynamic", sampler="its"), src, rings=(1, 2), ctas=(0,),
                           repeats=1)
        assert set(r4.timings) == {(0, 0), (1, 0), (2, 0), (-1, 0)}
        assert np.isfinite(list(r3.timings.values())).all()
        # the plain form as a tuned shape: same walks
        graph.set_engine_shape("alias", -1, 0)
        plain = E.compute(graph, src, app, seed=5)
        assert torch.equal(before.paths, plain.paths) and before.steps == plain.steps
        assert graph.engine_shape("alias") == (-1, 0)
    finally:
        graph.close()
