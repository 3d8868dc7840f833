"""Node2Vec's neighbour test through the edge set: on a directed graph (some
edges without their reverse) the reference's choice of list by degree
(graph.h:180-199) must be kept, and walks must equal the oracle's; on a
symmetric graph a single lookup decides."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu


def _directed_graph(n, m, seed):
    rng = np.random.default_rng(seed)
    # skewed out/in degrees so that the degree comparison matters
    u = (rng.pareto(1.2, m) * 3).astype(np.int64) % n
    v = rng.integers(0, n, m)
    keep = u != v
    pairs = np.unique(u[keep] * n + v[keep])
    src, dst = pairs // n, pairs % n
    row = np.zeros(n + 1, dtype=np.int64)
    np.add.at(row, src + 1, 1)
    np.cumsum(row, out=row)
    return row, dst.astype(np.int32)  # rows sorted: pairs are sorted by (src, dst)


@pytest.mark.parametrize("sampler", ["maxweight_rejection", "its", "alias", "rejection"])
def test_node2vec_directed_matches_oracle(sampler):
    torch, E = need_gpu()
    row, adj = _directed_graph(3000, 40000, seed=5)
    is_sym = set(zip(np.repeat(np.arange(3000), np.diff(row)).tolist(), adj.tolist()))
    assert any((b, a) not in is_sym for a, b in list(is_sym)[:2000])  # really directed
    og = O.Graph(row, adj)
    src = np.nonzero(np.diff(row))[0].astype(np.int32)
    d = O.make_desc("node2vec", "dynamic", sampler, length=16, p=2.0, q=0.5, seed=9)
    ref = O.walk(og, d, src, path_cap=16)
    g = E.Graph(row, adj, check_sorted=True)
    try:
        r = E.compute(g, src, E.Node2Vec(16, 2.0, 0.5, sampler=sampler), seed=9)
        np.testing.assert_array_equal(r.paths.cpu().numpy(), ref["paths"])
        np.testing.assert_array_equal(r.lengths.cpu().numpy(), ref["lengths"])
        assert r.steps == ref["steps"]
    finally:
        g.close()
