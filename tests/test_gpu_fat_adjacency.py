"""The adjacency with row pairs folded in (the uniform and max-weight
rejection moves' 16-byte entries) gives the walks of the plain layout: forced
on (TRW_FAT_ADJACENCY=1) and off (=0) for small graphs, the walks, counts and
steps equal the oracle's.  Large graphs take it by the L2 rule and are
covered by the config-scale tests."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture
def fat_env(monkeypatch):
    def set_mode(mode):
        monkeypatch.setenv("TRW_FAT_ADJACENCY", mode)
    return set_mode


@pytest.fixture(scope="module")
def rmat():
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 13, 16, seed=31, weights=False)
    return g["row"].numpy(), g["adj"].numpy()


def _directed(n, m, seed):
    rng = np.random.default_rng(seed)
    u = (rng.pareto(1.2, m) * 3).astype(np.int64) % n
    v = rng.integers(0, n, m)
    keep = u != v
    pairs = np.unique(u[keep] * n + v[keep])
    src, dst = pairs // n, pairs % n
    row = np.zeros(n + 1, dtype=np.int64)
    np.add.at(row, src + 1, 1)
    np.cumsum(row, out=row)
    return row, dst.astype(np.int32)


@pytest.mark.parametrize("mode", ["1", "0"])
def test_node2vec_paths(mode, fat_env, rmat):
    torch, E = need_gpu()
    fat_env(mode)
    for row, adj in (rmat, _directed(3000, 40000, seed=5)):
        og = O.Graph(row, adj)
        src = np.nonzero(np.diff(row))[0].astype(np.int32)
        d = O.make_desc("node2vec", "dynamic", "maxweight_rejection", length=24, p=2.0, q=0.5, seed=13)
        ref = O.walk(og, d, src, path_cap=24)
        g = E.Graph(row, adj)
        try:
            r = E.compute(g, src, E.Node2Vec(24, 2.0, 0.5), seed=13)
            np.testing.assert_array_equal(r.paths.cpu().numpy(), ref["paths"])
            np.testing.assert_array_equal(r.lengths.cpu().numpy(), ref["lengths"])
            assert r.steps == ref["steps"]
        finally:
            g.close()


@pytest.mark.parametrize("mode", ["1", "0"])
def test_ppr_uniform(mode, fat_env, rmat):
    torch, E = need_gpu()
    fat_env(mode)
    row, adj = rmat
    og = O.Graph(row, adj)
    rng = np.random.default_rng(3)
    qs = rng.choice(np.nonzero(np.diff(row))[0], 24, replace=False).astype(np.int32)
    ref = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=21), qs, per_query=500,
                 want_counts=True, want_lengths=False)
    g = E.Graph(row, adj)
    try:
        sp = E.ppr_batch_sparse(g, qs, 500, tp=0.2, seed=21)
        assert sp.steps == ref["steps"]
        assert torch.equal(sp.dense(g.n).cpu(), torch.from_numpy(ref["counts"]))
        # paths of single-source walks (the uniform move without visit tables)
        src = np.repeat(qs[:4], 64).astype(np.int32)
        d = O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=5)
        refp = O.walk(og, d, src, path_cap=64)
        r = E.compute(g, src, E.PPR(0.2), seed=5, path_cap=64)
        np.testing.assert_array_equal(r.paths.cpu().numpy(), refp["paths"])
        np.testing.assert_array_equal(r.lengths.cpu().numpy(), refp["lengths"])
    finally:
        g.close()


def _labelled():
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 12, 24, seed=61, labels=5)
    return g["row"].numpy(), g["adj"].numpy(), g["label"].numpy()


@pytest.mark.parametrize("mode", ["1", "0"])
def test_metapath_label_index_entries(mode, fat_env):
    """Schemas that name each label once read the label-index entries that
    carry the next step's block (forced on here); a schema with a repeated
    label, one with a label no edge has, and switching schemas on one graph
    (the entries are rebuilt) all give the oracle's walks."""
    torch, E = need_gpu()
    fat_env(mode)
    row, adj, lab = _labelled()
    w = np.ones(adj.size)
    src = np.nonzero(np.diff(row))[0].astype(np.int32)
    og = O.Graph(row, adj, w, lab)
    g = E.Graph(row, adj, w, lab)
    try:
        for schema, fat in (([0, 1, 2, 3, 4], True), ([3, 1, 4], True), ([2, 9, 1], True),
                            ([0, 1, 0, 2], False), ([0, 1, 2, 3, 4], True)):
            d = O.make_desc("metapath", "dynamic", "its", length=14, schema=schema, seed=23)
            ref = O.walk(og, d, src, path_cap=14, want_counts=True)
            r = E.compute(g, src, E.MetaPath(14, schema), seed=23, count_visits=True)
            np.testing.assert_array_equal(r.paths.cpu().numpy(), ref["paths"], err_msg=str(schema))
            np.testing.assert_array_equal(r.lengths.cpu().numpy(), ref["lengths"])
            np.testing.assert_array_equal(r.counts.cpu().numpy(), ref["counts"][0])
            assert r.steps == ref["steps"]
            state = g.layout()[1]
            if mode == "1" and fat:
                assert state == 1
            elif mode == "0":
                assert state == -1
    finally:
        g.close()
