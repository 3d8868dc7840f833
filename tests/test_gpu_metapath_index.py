"""MetaPath's label index (each row's neighbours stably sorted by label):
walks through it equal the oracle's row-scanning dynamic ITS; labels outside
[0, 64) keep the scan, with the same results."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu


def _graph():
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 12, 24, seed=61, labels=5)
    return g["row"].numpy(), g["adj"].numpy(), g["label"].numpy()


@pytest.mark.parametrize("labels,schema,want_state", [
    ("small", [0, 1, 2, 3, 4], 1),
    ("sparse", [0, 5, 63, 40, 0], 1),   # label ids with gaps, up to 63; 40 never occurs: walkers stop there
    ("large", [7, 1007, 2007, 3007], -1),  # outside [0, 64): the row scan stays
    ("negative", [-3, 0, 1, 2], -1),
])
def test_metapath_index_matches_oracle(labels, schema, want_state):
    torch, E = need_gpu()
    row, adj, lab = _graph()
    if labels == "sparse":
        lab = np.array([0, 5, 63, 17, 5], dtype=np.int32)[lab]
    elif labels == "large":
        lab = (lab * 1000 + 7).astype(np.int32)
    elif labels == "negative":
        lab = (lab - 3).astype(np.int32)
    w = np.ones(adj.size)
    src = np.nonzero(np.diff(row))[0].astype(np.int32)
    og = O.Graph(row, adj, w, lab)
    d = O.make_desc("metapath", "dynamic", "its", length=14, schema=schema, seed=21)
    ref = O.walk(og, d, src, path_cap=14, want_counts=True)
    g = E.Graph(row, adj, w, lab)
    try:
        assert g.indexes()[1] == 0
        for engine in ("persistent", "plain"):
            r = E.compute(g, src, E.MetaPath(14, schema), seed=21, count_visits=True, engine=engine)
            np.testing.assert_array_equal(r.paths.cpu().numpy(), ref["paths"])
            np.testing.assert_array_equal(r.lengths.cpu().numpy(), ref["lengths"])
            np.testing.assert_array_equal(r.counts.cpu().numpy(), ref["counts"][0])
            assert r.steps == ref["steps"]
        assert g.indexes()[1] == want_state
        if schema[3] == 40:  # the absent label stops walks: lengths of 4 entries occur
            assert (r.lengths.cpu().numpy() == 4).any()
    finally:
        g.close()


def test_build_indexes_up_front():
    """trw_graph_build_indexes builds the Node2Vec edge set and the MetaPath
    label index before any walk; walks then equal the oracle's (searching)
    walks, and a second build call changes nothing."""
    torch, E = need_gpu()
    row, adj, lab = _graph()
    w = np.ones(adj.size)
    src = np.nonzero(np.diff(row))[0].astype(np.int32)
    og = O.Graph(row, adj, w, lab)
    g = E.Graph(row, adj, w, lab)
    try:
        assert g.indexes() == (0, 0)
        assert g.build_indexes(edge_set=False, label_index=True) == (0, 1)
        assert g.build_indexes() == (1, 1)
        assert g.build_indexes() == (1, 1)
        cases = [(E.MetaPath(12, [0, 1, 2, 3, 4]), O.make_desc("metapath", "dynamic", "its", length=12,
                                                              schema=[0, 1, 2, 3, 4], seed=23)),
                 (E.Node2Vec(12, 2.0, 0.5), O.make_desc("node2vec", "dynamic", "maxweight_rejection", length=12,
                                                       p=2.0, q=0.5, seed=23))]
        for app, d in cases:
            ref = O.walk(og, d, src, path_cap=12)
            r = E.compute(g, src, app, seed=23)
            np.testing.assert_array_equal(r.paths.cpu().numpy(), ref["paths"])
            assert r.steps == ref["steps"]
        assert g.indexes() == (1, 1)
    finally:
        g.close()
