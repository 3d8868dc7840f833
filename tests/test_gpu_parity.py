"""CUDA engine vs the golden fixtures (reference samplers under shared
Philox uniforms) and vs the oracle on larger seeded graphs.  Everything runs
through the C ABI of libtrw_gpu.so; bit-exact equality is required (walks
and tables are integer / IEEE-double results of identical operation
sequences)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden_cases import CASES, case_arrays, case_id, graph_arrays
from tests.gpu_util import make_app, need_gpu, oracle_run, to_np

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("engine", ["persistent", "plain"])
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_golden_case(case, engine):
    torch, E = need_gpu()
    ga = graph_arrays(case["graph"])
    ref = case_arrays(case)
    g = E.Graph(ga["row"], ga["adj"], ga["weight"], ga["label"])
    try:
        if case["per_query"] > 0:
            counts, steps = E.ppr_batch(g, ref["sources"], case["per_query"], tp=case["tp"], seed=case["seed"],
                                        engine=engine)
            torch.cuda.synchronize()
            assert int(steps.item()) == case["steps"]
            np.testing.assert_array_equal(to_np(counts), ref["counts"])
            return
        res = E.compute(g, ref["sources"], make_app(E, case), seed=case["seed"], id_base=case["id_base"],
                        path_cap=case["path_cap"], count_visits=True, engine=engine)
        torch.cuda.synchronize()
        assert res.steps == case["steps"]
        np.testing.assert_array_equal(to_np(res.lengths), ref["lengths"])
        np.testing.assert_array_equal(to_np(res.paths), ref["paths"])
        np.testing.assert_array_equal(to_np(res.counts), ref["counts"][0])
        if case["mode"] == "static":
            tab = g.download_table(case["sampler"])
            key = {"alias": "alias", "its": "prefix", "rejection": "rejmax"}[case["sampler"]]
            assert tab.tobytes() == ref[key].tobytes()
        assert g.device_error() == 0
    finally:
        g.close()


COMBOS = [
    ("deepwalk", "static", "alias"), ("deepwalk", "static", "its"), ("deepwalk", "static", "rejection"),
    ("deepwalk", "uniform", "uniform"), ("deepwalk", "dynamic", "its"), ("deepwalk", "dynamic", "alias"),
    ("deepwalk", "dynamic", "rejection"), ("deepwalk", "dynamic", "maxweight_rejection"),
    ("ppr", "uniform", "uniform"), ("ppr", "static", "alias"), ("ppr", "static", "rejection"),
    ("ppr", "dynamic", "maxweight_rejection"), ("ppr", "dynamic", "its"),
    ("node2vec", "dynamic", "maxweight_rejection"), ("node2vec", "dynamic", "its"),
    ("node2vec", "dynamic", "alias"), ("node2vec", "dynamic", "rejection"),
    ("metapath", "dynamic", "its"), ("metapath", "dynamic", "alias"), ("metapath", "dynamic", "rejection"),
    ("genericwalk", "static", "its"),
]


@pytest.fixture(scope="module")
def rmat_hubs():
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 13, 16, seed=21, labels=5)
    return {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in g.items()}


@pytest.mark.parametrize("combo", COMBOS, ids=lambda c: "-".join(c))
def test_oracle_parity_hub_graph(rmat_hubs, combo):
    """R-MAT N=2^13 (hub rows of several hundred neighbours) against the oracle."""
    torch, E = need_gpu()
    from thunderrw_gb300 import generators as G
    app, mode, sm = combo
    L = 1 if app == "ppr" else 24
    case = dict(app=app, mode=mode, sampler=sm, length=max(L, 2), p=2.0, q=0.5, tp=0.15,
                schema=[0, 1, 2, 3, 4] if app == "metapath" else None, seed=1234, id_base=77, path_cap=L)
    src = G.all_sources(torch.from_numpy(rmat_hubs["row"]), seed=4).numpy()[:3000]
    _, ref = oracle_run(rmat_hubs, case, src)
    g = E.Graph(rmat_hubs["row"], rmat_hubs["adj"], rmat_hubs["weight"], rmat_hubs["label"])
    try:
        for engine in ("persistent", "plain"):
            res = E.compute(g, src, make_app(E, case), seed=1234, id_base=77, path_cap=L, count_visits=True,
                            engine=engine)
            torch.cuda.synchronize()
            assert res.steps == ref["steps"], engine
            np.testing.assert_array_equal(to_np(res.paths), ref["paths"])
            np.testing.assert_array_equal(to_np(res.lengths), ref["lengths"])
            np.testing.assert_array_equal(to_np(res.counts), ref["counts"][0])
    finally:
        g.close()


@pytest.mark.parametrize("ring", [1, 2, 4, 8])
@pytest.mark.parametrize("sampler", ["alias", "its", "rejection"])
def test_ring_depths_and_occupancy(rmat_hubs, ring, sampler):
    """Every launch shape of the persistent engine walks identically."""
    torch, E = need_gpu()
    from thunderrw_gb300 import generators as G
    case = dict(app="deepwalk", mode="static", sampler=sampler, length=30, p=1, q=1, tp=0.2, schema=None,
                seed=5, id_base=0, path_cap=30)
    src = G.all_sources(torch.from_numpy(rmat_hubs["row"]), seed=8).numpy()
    _, ref = oracle_run(rmat_hubs, case, src, counts=False)
    g = E.Graph(rmat_hubs["row"], rmat_hubs["adj"], rmat_hubs["weight"], rmat_hubs["label"])
    try:
        for ctas in (0, 1):
            g.set_engine_shape(sampler, ring, ctas)
            assert g.engine_shape(sampler) == (ring, ctas)
            res = E.compute(g, src, E.DeepWalk(30, sampler=sampler), seed=5)
            np.testing.assert_array_equal(to_np(res.paths), ref["paths"])
            assert res.steps == ref["steps"]
    finally:
        g.close()


def test_table_builders_match_oracle(rmat_hubs):
    torch, E = need_gpu()
    og = O.Graph(rmat_hubs["row"], rmat_hubs["adj"], rmat_hubs["weight"])
    g = E.Graph(rmat_hubs["row"], rmat_hubs["adj"], rmat_hubs["weight"])
    try:
        for kind, wk in (("edge", 0), ("unit", 1)):
            for sm in ("alias", "its", "rejection"):
                og.build_tables(sm, wk)
                g.build_tables(sm, kind)
                tab = g.download_table(sm)
                want = {"alias": og.alias, "its": og.prefix, "rejection": og.rej_max}[sm]
                assert tab.tobytes() == want.tobytes(), (sm, kind)
    finally:
        g.close()


def test_ppr_batch_matches_oracle(rmat_hubs):
    torch, E = need_gpu()
    from thunderrw_gb300 import generators as G
    qs = G.random_sources(torch.from_numpy(rmat_hubs["row"]), 37, seed=2).numpy()
    og = O.Graph(rmat_hubs["row"], rmat_hubs["adj"])
    ref = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=99), qs, per_query=500,
                 want_counts=True, want_lengths=False)
    g = E.Graph(rmat_hubs["row"], rmat_hubs["adj"])
    try:
        for engine in ("persistent", "plain"):
            counts, steps = E.ppr_batch(g, qs, 500, tp=0.2, seed=99, engine=engine)
            assert int(steps.item()) == ref["steps"]
            np.testing.assert_array_equal(to_np(counts), ref["counts"])
        # accumulate mode: a second batch adds to the first
        counts2, _ = E.ppr_batch(g, qs, 500, tp=0.2, seed=99, counts=counts.clone(), zero_counts=False)
        np.testing.assert_array_equal(to_np(counts2), 2 * ref["counts"])
    finally:
        g.close()


def test_host_pointer_staging(rmat_hubs):
    """Host (numpy) buffers through the raw C ABI: the library stages them."""
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    L = N.load()
    row, adj, w = rmat_hubs["row"], rmat_hubs["adj"], rmat_hubs["weight"]
    h = ctypes.c_void_p()
    N.check(L.trw_graph_create(row.ctypes.data, adj.ctypes.data, w.ctypes.data, None, row.size - 1, adj.size, 1,
                               ctypes.byref(h)))
    try:
        src = np.ascontiguousarray(np.nonzero(np.diff(row))[0][:1000].astype(np.int32))
        paths = np.zeros((src.size, 20), dtype=np.int32)
        lengths = np.zeros(src.size, dtype=np.int32)
        counts = np.zeros(row.size - 1, dtype=np.int32)
        steps = np.zeros(1, dtype=np.uint64)
        d = E.DeepWalk(20).desc(3)
        N.check(L.trw_walk(h, ctypes.byref(d), src.ctypes.data, src.size, 0, paths.ctypes.data, 20,
                           lengths.ctypes.data, counts.ctypes.data, steps.ctypes.data, 0, None))
        og = O.Graph(row, adj, w)
        og.build_tables("alias", 0)
        ref = O.walk(og, O.make_desc("deepwalk", "static", "alias", length=20, seed=3), src, path_cap=20,
                     want_counts=True)
        assert int(steps[0]) == ref["steps"]
        np.testing.assert_array_equal(paths, ref["paths"])
        np.testing.assert_array_equal(lengths, ref["lengths"])
        np.testing.assert_array_equal(counts, ref["counts"][0])
    finally:
        L.trw_graph_destroy(h)


def test_sinks_and_directed_rows():
    """A non-symmetric CSR with out-degree-0 vertices: walkers stop there."""
    torch, E = need_gpu()
    rng = np.random.default_rng(3)
    n = 600
    deg = rng.integers(0, 6, size=n)
    row = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg, out=row[1:])
    adj = np.concatenate([np.sort(rng.choice(n, size=d, replace=False)) for d in deg]).astype(np.int32)
    w = rng.random(adj.size) + 0.01
    src = np.nonzero(deg)[0].astype(np.int32)
    for mode, sm in (("static", "alias"), ("uniform", "uniform"), ("static", "its"), ("dynamic", "its")):
        case = dict(app="deepwalk", mode=mode, sampler=sm, length=15, p=1, q=1, tp=0.2, schema=None, seed=8,
                    path_cap=15)
        _, ref = oracle_run({"row": row, "adj": adj, "weight": w}, case, src)
        g = E.Graph(row, adj, w)
        res = E.compute(g, src, make_app(E, case), seed=8, count_visits=True)
        assert res.steps == ref["steps"]
        np.testing.assert_array_equal(to_np(res.paths), ref["paths"])
        np.testing.assert_array_equal(to_np(res.lengths), ref["lengths"])
        g.close()


def test_error_behaviour(rmat_hubs):
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    g = E.Graph(rmat_hubs["row"], rmat_hubs["adj"], rmat_hubs["weight"], rmat_hubs["label"])
    try:
        with pytest.raises(N.TrwError) as ei:
            E.compute(g, [0, 1], E.Node2Vec(10, mode="static", sampler="alias"))
        assert ei.value.code == -3
        with pytest.raises(N.TrwError) as ei:
            E.compute(g, [0, 1], E.MetaPath(10, sampler="maxweight_rejection"))
        assert ei.value.code == -3
        with pytest.raises(N.TrwError) as ei:
            E.compute(g, [0, 1], E.DeepWalk(1))
        assert ei.value.code == -1
        with pytest.raises(N.TrwError):
            E.compute(g, [0, 1], E.PPR(0.0))
        # an out-of-range source is reported, not read
        res = E.compute(g, [0, g.n + 5], E.DeepWalk(5), count_visits=True)
        torch.cuda.synchronize()
        assert g.device_error() == 2
        assert int(res.lengths[1].item()) == 1
        # empty walker set
        res = E.compute(g, np.zeros(0, dtype=np.int32), E.DeepWalk(5))
        assert res.steps == 0
    finally:
        g.close()
    with pytest.raises(N.TrwError) as ei:
        E.Graph(np.array([0, 2, 1], dtype=np.int64), np.array([1, 0], dtype=np.int32))
    assert ei.value.code == -5
