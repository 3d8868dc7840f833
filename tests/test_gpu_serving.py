"""The request loop: a mix of apps and sizes submitted while others run gives
every request exactly the result it gets alone; admission respects the HBM
budget; latency statistics are reported."""
import numpy as np
import pytest

from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph_arrays():
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 13, 16, seed=41, labels=5)
    return {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in g.items()}


def _requests(rng, n, deg):
    nz = np.nonzero(deg)[0].astype(np.int32)
    out = []
    for i in range(30):
        kind = ["deepwalk", "node2vec", "metapath", "ppr", "ppr1"][i % 5]
        walkers = int(rng.integers(200, 6000))
        src = rng.choice(nz, size=3 if kind == "ppr" else 1 if kind == "ppr1" else walkers)
        out.append(dict(kind=kind, walkers=walkers, length=int(rng.integers(5, 40)), seed=100 + i, src=src))
    return out


def _alone(E, graph, reqs, app_of):
    out = []
    for r in reqs:
        if r["kind"] in ("ppr", "ppr1"):
            sp = E.ppr_batch_sparse(graph, r["src"], r["walkers"], tp=0.2, seed=r["seed"])
            total = int(sp.offsets[-1].item())
            out.append((sp.offsets.cpu().numpy(), sp.vertices[:total].cpu().numpy(),
                        sp.counts[:total].cpu().numpy(), sp.steps))
        else:
            res = E.compute(graph, r["src"], app_of(r), seed=r["seed"])
            out.append((res.paths.cpu().numpy(), res.lengths.cpu().numpy(), res.steps))
    return out


def _check(srv, reqs, tickets, alone):
    for r, t, a in zip(reqs, tickets, alone):
        got = srv.result(t)
        if r["kind"] in ("ppr", "ppr1"):
            np.testing.assert_array_equal(got["offsets"], a[0])
            np.testing.assert_array_equal(got["vertices"], a[1])
            np.testing.assert_array_equal(got["counts"], a[2])
            assert got["steps"] == a[3]
        else:
            np.testing.assert_array_equal(got["paths"], a[0])
            np.testing.assert_array_equal(got["lengths"], a[1])
            assert got["steps"] == a[2]
        srv.release(t)


def test_mix_equals_alone(graph_arrays):
    torch, E = need_gpu()
    from thunderrw_gb300.serving import Server
    g = graph_arrays
    graph = E.Graph(g["row"], g["adj"], g["weight"], g["label"])
    graph.build_tables("alias", "edge")
    rng = np.random.default_rng(7)
    reqs = _requests(rng, graph.n, np.diff(g["row"]))

    def app_of(r):
        return {"deepwalk": E.DeepWalk(r["length"]), "node2vec": E.Node2Vec(r["length"], 2.0, 0.5),
                "metapath": E.MetaPath(r["length"], [0, 1, 2, 3, 4])}[r["kind"]]

    alone = []
    for r in reqs:
        if r["kind"] in ("ppr", "ppr1"):
            sp = E.ppr_batch_sparse(graph, r["src"], r["walkers"], tp=0.2, seed=r["seed"])
            total = int(sp.offsets[-1].item())
            alone.append((sp.offsets.cpu().numpy(), sp.vertices[:total].cpu().numpy(),
                          sp.counts[:total].cpu().numpy(), sp.steps))
        else:
            res = E.compute(graph, r["src"], app_of(r), seed=r["seed"])
            alone.append((res.paths.cpu().numpy(), res.lengths.cpu().numpy(), res.steps))
    torch.cuda.synchronize()

    # a budget that holds only a few requests at a time: the rest wait for memory
    srv = Server(graph, hbm_budget_bytes=6 << 20, max_inflight=4)
    try:
        tickets = []
        for r in reqs:
            if r["kind"] in ("ppr", "ppr1"):
                tickets.append(srv.submit_ppr(r["src"], r["walkers"], tp=0.2, seed=r["seed"]))
            else:
                tickets.append(srv.submit_walk(app_of(r), r["src"], seed=r["seed"]))
        for r, t, a in zip(reqs, tickets, alone):
            got = srv.result(t)
            if r["kind"] in ("ppr", "ppr1"):
                np.testing.assert_array_equal(got["offsets"], a[0])
                np.testing.assert_array_equal(got["vertices"], a[1])
                np.testing.assert_array_equal(got["counts"], a[2])
                assert got["steps"] == a[3]
            else:
                np.testing.assert_array_equal(got["paths"], a[0])
                np.testing.assert_array_equal(got["lengths"], a[1])
                assert got["steps"] == a[2]
            srv.release(t)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["steps"] == sum(a[-1] for a in alone)
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
        assert st["hbm_in_use"] == 0
    finally:
        srv.stop()
        graph.close()


def test_request_above_budget_is_refused(graph_arrays):
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300.serving import Server
    g = graph_arrays
    graph = E.Graph(g["row"], g["adj"], g["weight"], g["label"])
    srv = Server(graph, hbm_budget_bytes=1 << 16, max_inflight=2)
    try:
        with pytest.raises(N.TrwError) as ei:
            srv.submit_walk(E.DeepWalk(80), np.zeros(5000, dtype=np.int32))
        assert ei.value.code == -7
    finally:
        srv.stop()
        graph.close()


def test_requests_share_launches(graph_arrays):
    """With room for everything, requests submitted together go into few
    batches (one persistent launch per kernel of each batch, the walkers of
    all its requests on one work queue), and every result is still the one
    the request gets alone."""
    torch, E = need_gpu()
    from thunderrw_gb300.serving import Server
    g = graph_arrays
    graph = E.Graph(g["row"], g["adj"], g["weight"], g["label"])
    graph.build_tables("alias", "edge")
    graph.build_indexes()
    rng = np.random.default_rng(8)
    reqs = _requests(rng, graph.n, np.diff(g["row"]))

    def app_of(r):
        return {"deepwalk": E.DeepWalk(r["length"]), "node2vec": E.Node2Vec(r["length"], 2.0, 0.5),
                "metapath": E.MetaPath(r["length"], [0, 1, 2, 3, 4])}[r["kind"]]

    alone = _alone(E, graph, reqs, app_of)
    torch.cuda.synchronize()
    srv = Server(graph, max_inflight=2)
    try:
        tickets = []
        for r in reqs:
            if r["kind"] in ("ppr", "ppr1"):
                tickets.append(srv.submit_ppr(r["src"], r["walkers"], tp=0.2, seed=r["seed"]))
            else:
                tickets.append(srv.submit_walk(app_of(r), r["src"], seed=r["seed"]))
        _check(srv, reqs, tickets, alone)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["batches"] < len(reqs)
    finally:
        srv.stop()
        graph.close()
