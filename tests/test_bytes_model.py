"""The roofline's byte model (thunderrw_gb300/bytes_model.py) against the
oracle's sector-counting pass over the same walks."""
import numpy as np
import pytest

from oracle import oracle as O
from thunderrw_gb300 import bytes_model as B
from thunderrw_gb300 import generators as G


def _aligned(a, dtype):
    """A copy of `a` whose data starts on a 64-byte boundary (sector
    accounting depends on it)."""
    a = np.asarray(a, dtype=dtype)
    buf = np.empty(a.nbytes + 64, dtype=np.uint8)
    off = (-buf.ctypes.data) % 64
    out = buf[off:off + a.nbytes].view(dtype)
    out[...] = a
    return out


@pytest.fixture(scope="module")
def graph():
    g = G.make_graph("rmat", 1 << 11, 10, seed=31, labels=3)
    return O.Graph(_aligned(g["row"], np.int64), _aligned(g["adj"], np.int32), _aligned(g["weight"], np.float64),
                   _aligned(g["label"], np.int32))


def test_node2vec_model_equals_probe_accounting(graph):
    src = np.nonzero(np.diff(graph.row))[0][:1500].astype(np.int32)
    d = O.make_desc("node2vec", "dynamic", "maxweight_rejection", length=12, p=1.0, q=1.0, seed=3)  # no rejections
    walks = O.walk(graph, d, src, path_cap=12)
    nb, ns = O.count_bytes(graph, d, src, record_paths=True, neighbor_probe=True)
    assert ns == walks["steps"]
    assert B.node2vec(walks["paths"], 12) == pytest.approx(nb / ns, rel=1e-12)
    # with rejections (p = 2, q = 0.5) the model charges accepted moves only: a lower bound
    d2 = O.make_desc("node2vec", "dynamic", "maxweight_rejection", length=12, p=2.0, q=0.5, seed=3)
    w2 = O.walk(graph, d2, src, path_cap=12)
    nb2, ns2 = O.count_bytes(graph, d2, src, record_paths=True, neighbor_probe=True)
    assert B.node2vec(w2["paths"], 12) <= nb2 / ns2
    # the reference's binary search costs more than one probe
    nb3, _ = O.count_bytes(graph, d2, src, record_paths=True, neighbor_probe=False)
    assert nb3 > nb2


def test_metapath_model_equals_oracle(graph):
    src = np.nonzero(np.diff(graph.row))[0][:1500].astype(np.int32)
    d = O.make_desc("metapath", "dynamic", "its", length=10, schema=[0, 1, 2], seed=4)
    walks = O.walk(graph, d, src, path_cap=10)
    nb, ns = O.count_bytes(graph, d, src, record_paths=True)
    assert (walks["lengths"] < 10).any()  # some walks stop on rows without the label
    assert B.metapath(walks["paths"], graph.row, 10) == pytest.approx(nb / ns, rel=1e-12)


def test_metapath_index_model_equals_oracle(graph):
    src = np.nonzero(np.diff(graph.row))[0][:1500].astype(np.int32)
    d = O.make_desc("metapath", "dynamic", "its", length=10, schema=[0, 1, 2], seed=4)
    walks = O.walk(graph, d, src, path_cap=10)
    nb, ns = O.count_bytes(graph, d, src, record_paths=True, label_index=True)
    assert B.metapath_index(walks["paths"], graph.row, 10) == pytest.approx(nb / ns, rel=1e-12)
    # label-index entries carrying the next block: one sector and the path
    # entry per move, plus each walker's source positions; no stop charge
    moves = int(((walks["paths"][:, :-1] >= 0) & (walks["paths"][:, 1:] >= 0)).sum())
    fat = B.metapath_index(walks["paths"], graph.row, 10, fat=True)
    assert fat * moves == pytest.approx(moves * 36 + 32 * src.size)
    assert fat < B.metapath_index(walks["paths"], graph.row, 10)


def test_constant_models(graph):
    src = np.nonzero(np.diff(graph.row))[0][:800].astype(np.int32)
    graph.build_tables("alias", 0)
    d = O.make_desc("deepwalk", "static", "alias", length=10, seed=5)
    nb, ns = O.count_bytes(graph, d, src, record_paths=True)
    assert nb / ns == B.STATIC_ALIAS
    d = O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=6)
    nb, ns = O.count_bytes(graph, d, src, per_query=20, record_paths=False, count_visits=True)
    assert nb / ns == B.UNIFORM_PPR


def test_sector_reuse_counts_hot_sectors():
    """Walks that all leave one source through its one neighbour: the
    source's row-pair sector and the neighbour's adjacency sector take a
    large share of the reads, and an L2-sized cache holds every sector."""
    from thunderrw_gb300 import bytes_model as B
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 12, 8, seed=3, weights=False)
    row, adj = g["row"].numpy(), g["adj"].numpy()
    og = O.Graph(row, adj)
    src = np.full(64, int(np.argmax(np.diff(row))), dtype=np.int32)
    r = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=3), src, per_query=100,
               path_cap=32)
    out = B.sector_reuse(r["paths"], row, adj, cache_bytes=(1024, 129 << 20))
    assert out["moves"] > 0
    assert out["row_pair_hit_132096KB"] == 1.0 and out["adjacency_hit_132096KB"] == 1.0
    assert 0.0 < out["row_pair_hit_1KB"] <= 1.0
    share = B.top_degree_share(r["paths"], row, ks=(1, 4096))
    assert share[4096] == 1.0 and share[1] > 0.0  # every walk starts at the highest-degree vertex


def test_philox_restatement_matches_oracle():
    """The byte model's vectorised Philox4x32-10 gives the oracle's words."""
    from thunderrw_gb300 import bytes_model as B
    for seed, w, st, blk in [(1, 0, 1, 0), (12345678901, 77, 5, 0), (2**63 + 5, 2**33 + 9, 79, 3),
                             (7, 1 << 20, 2, 0x80000000)]:
        ref = O.philox([blk, st, w & 0xFFFFFFFF, w >> 32], [seed & 0xFFFFFFFF, seed >> 32])
        got = [int(B.philox_word(seed, np.array([w]), np.array([st]), blk, i)[0]) for i in range(4)]
        assert got == [int(x) for x in ref]
    assert B.accept_threshold(2.0, 1.0) == 1 << 31
    assert B.accept_threshold(2.0, 2.0) == 0xFFFFFFFF


def test_node2vec_model_charges_probes_only_in_the_band():
    """With the seed, moves whose first acceptance draw lies at or below the
    lower threshold are not charged a probe: fewer bytes than the plain count."""
    from thunderrw_gb300 import bytes_model as B
    g = G.make_graph("rmat", 1 << 11, 8, seed=4, weights=False)
    og = O.Graph(g["row"].numpy(), g["adj"].numpy())
    src = G.all_sources(g["row"], seed=1).numpy()[:500]
    r = O.walk(og, O.make_desc("node2vec", "dynamic", "maxweight_rejection", length=20, p=2.0, q=0.5, seed=9), src,
               path_cap=20)
    full = B.node2vec(r["paths"], 20)
    lazy = B.node2vec(r["paths"], 20, seed=9, p=2.0, q=0.5)
    assert 68.0 < lazy < full
    # with row pairs in the adjacency entries: one sector less per move, but
    # each walker's source row pair
    fat = B.node2vec(r["paths"], 20, seed=9, p=2.0, q=0.5, fat=True)
    moves = int(((r["paths"][:, :-1] >= 0) & (r["paths"][:, 1:] >= 0)).sum())
    first = int((r["paths"][:, 1] >= 0).sum())
    stops = B._stops(r["paths"], 20).size
    assert fat * moves == pytest.approx(lazy * moves - 32 * moves + 32 * first - 32 * stops)
