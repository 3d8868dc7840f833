"""Parity at the benchmark configurations' full sizes.

The golden fixtures pin the samplers on graphs of a few hundred vertices.
These tests run the benchmark's own graphs (the seeded generators of
bench.py: Chung-Lu 2^18, R-MAT 2^22, R-MAT 2^24 with and without labels)
through the C ABI at full size and compare with the CPU oracle bit for bit:

* DeepWalk, static alias (Chung-Lu N = 2^18, degree 16, one walker per
  vertex, L = 80): the whole alias table (its hub row has ~61 K entries and
  is built by the warp builder) and every path (alias_sampling.h:12-54,
  147-172);
* batched PPR (R-MAT N = 2^22, degree 32, 4096 queries x 10^4 walkers,
  tp = 0.2): the whole batch in one call; every query's visit counts sum to
  the batch's steps, and the (vertex, count) lists of query ranges at the
  start, middle and end of the batch equal the oracle's
  (uniform_sampling.h:47-63, ppr.cpp:22-34);
* Node2Vec, dynamic max-weight rejection (R-MAT N = 2^24, degree 16, one
  walker per vertex, L = 80) with the edge set built: the whole batch,
  walker ranges at the start, middle and end (rejection_sampling.h:368-402,
  node2vec.cpp:9-47, graph.h:180-199);
* MetaPath, dynamic ITS (R-MAT N = 2^24, degree 32, 5 labels, 2^22 random
  sources, L = 20) with the label index built: the whole batch, walker
  ranges at the start, middle and end (inverse_transformation_sampling.h:
  288-313, metapath.cpp:9-39).

Walker ids are batch indexes, so a range of the GPU's full batch equals the
oracle's walk of that range with id_base = its first index.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu
from tests.sparse_order import canonical, table_bits

pytestmark = pytest.mark.gpu

FULL = SimpleNamespace(scale=None, queries=None)
RANGE = 1 << 13  # walkers per compared range


def _inputs(name):
    torch, E = need_gpu()
    import bench
    wl = bench.WORKLOADS[name]
    inp = bench.build_inputs(wl, FULL, "cuda")
    host = bench.host_arrays(inp)
    return torch, E, wl, inp, host


def _ranges(total, width=RANGE):
    mid = max(0, total // 2 - width // 2)
    out = []
    for a in (0, mid, max(0, total - width)):
        b = min(total, a + width)
        if (a, b) not in out:
            out.append((a, b))
    return out


def test_deepwalk_chunglu_2e18_full():
    torch, E, wl, inp, host = _inputs("deepwalk")
    g = E.Graph(inp["row"], inp["adj"], inp["weight"])
    try:
        assert g.max_degree_ > 32 * 1024  # the hub row goes to the warp builder
        og = O.Graph(host["row"], host["adj"], host["weight"])
        og.build_tables("alias", 0)
        g.build_tables("alias", "edge")
        table = g.download_table("alias")
        assert table.tobytes() == og.alias.tobytes()
        src = inp["sources"]
        L = wl["length"]
        res = E.compute(g, src, E.DeepWalk(L), seed=1)
        torch.cuda.synchronize()
        ref = O.walk(og, O.make_desc("deepwalk", "static", "alias", length=L, seed=1), host["sources"], path_cap=L)
        assert res.steps == ref["steps"] == src.numel() * (L - 1)
        assert np.array_equal(res.paths.cpu().numpy(), ref["paths"])
        assert np.array_equal(res.lengths.cpu().numpy(), ref["lengths"])
        assert g.device_error() == 0
    finally:
        g.close()


def test_ppr_batch_rmat_2e22_full_batch():
    torch, E, wl, inp, host = _inputs("ppr")
    g = E.Graph(inp["row"], inp["adj"])
    try:
        src = inp["sources"]
        Q, pq, tp = src.numel(), wl["per_query"], wl["tp"]
        assert Q == 4096 and pq == 10_000
        sp = E.ppr_batch_sparse(g, src, pq, tp=tp, seed=123)
        off = sp.offsets.cpu().numpy()
        vert = sp.vertices[: off[-1]].cpu().numpy()
        cnt = sp.counts[: off[-1]].cpu().numpy()
        # every move is one visit: the counts of the whole batch sum to its steps
        assert int(cnt.astype(np.int64).sum()) == sp.steps
        assert np.all(np.diff(off) > 0) and np.all(cnt > 0)
        assert vert.min() >= 0 and vert.max() < g.n
        og = O.Graph(host["row"], host["adj"])
        d = O.make_desc("ppr", "uniform", "uniform", length=1, tp=tp, seed=123)
        bits = table_bits(pq, tp, g.n)
        assert bits == 16
        for a, b in _ranges(Q, 24):
            ref = O.walk(og, d, host["sources"][a:b], per_query=pq, id_base=a * pq, want_counts=True,
                         want_lengths=False)
            for q in range(a, b):
                v, c = vert[off[q]:off[q + 1]], cnt[off[q]:off[q + 1]]
                assert np.unique(v).size == v.size, q
                nz = np.nonzero(ref["counts"][q - a])[0]
                order = np.argsort(v)
                assert np.array_equal(v[order], nz), q
                assert np.array_equal(c[order], ref["counts"][q - a][nz]), q
                # the emit's canonical order on the full-size (2^16-slot) table
                assert np.array_equal(v, canonical(v, bits)), q
        assert g.device_error() == 0
    finally:
        g.close()


def _walk_ranges(torch, E, g, app, inp, host, desc, L, check_index):
    src = inp["sources"]
    W = src.numel()
    res = E.compute(g, src, app, seed=desc.seed)
    torch.cuda.synchronize()
    assert check_index(g.indexes())
    paths = res.paths
    lengths = res.lengths
    og = O.Graph(host["row"], host["adj"], host["weight"], host["label"])
    for a, b in _ranges(W):
        ref = O.walk(og, desc, host["sources"][a:b], id_base=a, path_cap=L)
        assert np.array_equal(paths[a:b].cpu().numpy(), ref["paths"]), (a, b)
        assert np.array_equal(lengths[a:b].cpu().numpy(), ref["lengths"]), (a, b)
    assert g.device_error() == 0
    return res


def test_node2vec_rmat_2e24_full_batch():
    torch, E, wl, inp, host = _inputs("node2vec")
    g = E.Graph(inp["row"], inp["adj"], inp["weight"])
    try:
        L = wl["length"]
        app = E.Node2Vec(L, wl["p"], wl["q"])
        desc = O.make_desc("node2vec", "dynamic", "maxweight_rejection", length=L, p=wl["p"], q=wl["q"], seed=31)
        res = _walk_ranges(torch, E, g, app, inp, host, desc, L, lambda ix: ix[0] == 1)  # edge set built
        assert res.steps == inp["sources"].numel() * (L - 1)
    finally:
        g.close()


def test_metapath_rmat_2e24_full_batch():
    torch, E, wl, inp, host = _inputs("metapath")
    g = E.Graph(inp["row"], inp["adj"], inp["weight"], inp["label"])
    try:
        L = wl["length"]
        app = E.MetaPath(L, wl["schema"])
        desc = O.make_desc("metapath", "dynamic", "its", length=L, schema=wl["schema"], seed=41)
        _walk_ranges(torch, E, g, app, inp, host, desc, L, lambda ix: ix[1] == 1)  # label index built
    finally:
        g.close()
