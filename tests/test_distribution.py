"""Chi-square tests of the sampled transitions against exact probabilities.

Bit parity with the reference samplers is checked elsewhere; these tests pin
the distributions themselves: w_i / sum(w) for alias, ITS and rejection
(static and dynamic), the second-order Node2Vec law (1/p back, 1 to common
neighbours, 1/q elsewhere), MetaPath's uniform choice among label matches and
PPR's geometric walk lengths.  The CPU tests sample through the oracle, the
GPU tests through the CUDA engine.  Seeds are fixed, so the p-values are
deterministic; the threshold 1e-6 only catches a wrong law.
"""
import numpy as np
import pytest

scipy_stats = pytest.importorskip("scipy.stats")

from oracle import oracle as O  # noqa: E402
from thunderrw_gb300 import generators as G  # noqa: E402

P_MIN = 1e-6


@pytest.fixture(scope="module")
def graph():
    g = G.make_graph("rmat", 1 << 11, 14, seed=31, labels=3)
    return {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in g.items()}


def _hub(g, rank=3):
    deg = np.diff(g["row"])
    return int(np.argsort(deg)[-rank])


def _chisq(observed, expected):
    observed = np.asarray(observed, dtype=np.float64)
    expected = np.asarray(expected, dtype=np.float64)
    keep = expected >= 5
    obs = np.append(observed[keep], observed[~keep].sum())
    exp = np.append(expected[keep], expected[~keep].sum())
    if exp[-1] == 0:
        obs, exp = obs[:-1], exp[:-1]
    exp = exp * obs.sum() / exp.sum()
    return scipy_stats.chisquare(obs, exp).pvalue


def _first_step_expected(g, v, weights):
    lo, hi = g["row"][v], g["row"][v + 1]
    nb = g["adj"][lo:hi]
    w = weights[lo:hi]
    return nb, w / w.sum()


def _sample_first_steps(walk_fn, v, W):
    paths = walk_fn(np.full(W, v, dtype=np.int32))
    return paths[:, 1]


def _oracle_walker(g, app, mode, sampler, L, **kw):
    og = O.Graph(g["row"], g["adj"], g["weight"], g["label"])
    if mode == "static":
        og.build_tables(sampler, 1 if app == "ppr" else 0)
    d = O.make_desc(app, mode, sampler, length=L, seed=kw.pop("seed", 17), **kw)
    return lambda src: O.walk(og, d, src, path_cap=L)["paths"]


SAMPLERS = [("static", "alias"), ("static", "its"), ("static", "rejection"), ("dynamic", "its"),
            ("dynamic", "alias"), ("dynamic", "rejection"), ("dynamic", "maxweight_rejection")]


@pytest.mark.parametrize("mode,sampler", SAMPLERS)
def test_weighted_first_step_oracle(graph, mode, sampler):
    v = _hub(graph)
    nb, p = _first_step_expected(graph, v, graph["weight"])
    nxt = _sample_first_steps(_oracle_walker(graph, "deepwalk", mode, sampler, 2), v, 200_000)
    obs = np.array([(nxt == x).sum() for x in nb])
    assert obs.sum() == nxt.size
    assert _chisq(obs, p * nxt.size) > P_MIN


def test_uniform_first_step_oracle(graph):
    v = _hub(graph)
    nb, p = _first_step_expected(graph, v, np.ones(graph["adj"].size))
    nxt = _sample_first_steps(_oracle_walker(graph, "deepwalk", "uniform", "uniform", 2), v, 100_000)
    assert _chisq([(nxt == x).sum() for x in nb], p * nxt.size) > P_MIN


def _node2vec_pairs(g, u, p, q):
    """Exact law of (x1, x2) for a walker starting at u."""
    row, adj = g["row"], g["adj"]
    n_u = set(adj[row[u]:row[u + 1]].tolist())
    pairs, probs = [], []
    d1 = row[u + 1] - row[u]
    for v in adj[row[u]:row[u + 1]]:
        nb = adj[row[v]:row[v + 1]]
        w = np.array([1.0 / p if x == u else (1.0 if x in n_u else 1.0 / q) for x in nb])
        for x, wx in zip(nb, w / w.sum()):
            pairs.append((int(v), int(x)))
            probs.append(wx / d1)
    return pairs, np.array(probs)


def _pair_counts(paths, pairs):
    key = paths[:, 1].astype(np.int64) * (1 << 32) + paths[:, 2]
    uniq, cnt = np.unique(key, return_counts=True)
    lut = dict(zip(uniq.tolist(), cnt.tolist()))
    return np.array([lut.get(a * (1 << 32) + b, 0) for a, b in pairs])


def test_node2vec_second_order_oracle(graph):
    u = _hub(graph, rank=40)
    pairs, probs = _node2vec_pairs(graph, u, 2.0, 0.5)
    walk = _oracle_walker(graph, "node2vec", "dynamic", "maxweight_rejection", 3, p=2.0, q=0.5)
    paths = walk(np.full(300_000, u, dtype=np.int32))
    obs = _pair_counts(paths, pairs)
    assert obs.sum() == paths.shape[0]
    assert _chisq(obs, probs * paths.shape[0]) > P_MIN


def test_metapath_label_filter_oracle(graph):
    v = _hub(graph)
    schema = [1, 0, 2]
    lo, hi = graph["row"][v], graph["row"][v + 1]
    match = graph["label"][lo:hi] == schema[0]
    nb = graph["adj"][lo:hi][match]
    walk = _oracle_walker(graph, "metapath", "dynamic", "its", 2, schema=schema)
    nxt = walk(np.full(100_000, v, dtype=np.int32))[:, 1]
    assert set(np.unique(nxt).tolist()) <= set(nb.tolist())
    assert _chisq([(nxt == x).sum() for x in nb], np.full(nb.size, nxt.size / nb.size)) > P_MIN


def test_ppr_lengths_geometric_oracle(graph):
    og = O.Graph(graph["row"], graph["adj"])
    tp = 0.2
    src = G.all_sources(__import__("torch").from_numpy(graph["row"]), seed=2).numpy()
    src = np.resize(src, 200_000).astype(np.int32)
    r = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=tp, seed=5), src, path_cap=0)
    moves = r["lengths"] - 1
    assert moves.min() >= 1
    k = np.arange(1, 30)
    expected = (1 - tp) ** (k - 1) * tp
    obs = np.array([(moves == x).sum() for x in k])
    assert _chisq(np.append(obs, (moves >= 30).sum()),
                  np.append(expected, (1 - tp) ** 29) * moves.size) > P_MIN


# ---------------------------------------------------------------------------
# the same laws on the GPU engine
# ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("mode,sampler", SAMPLERS)
def test_weighted_first_step_gpu(graph, mode, sampler):
    from tests.gpu_util import need_gpu
    torch, E = need_gpu()
    g = E.Graph(graph["row"], graph["adj"], graph["weight"], graph["label"])
    try:
        v = _hub(graph)
        nb, p = _first_step_expected(graph, v, graph["weight"])
        res = E.compute(g, np.full(400_000, v, dtype=np.int32), E.DeepWalk(2, mode=mode, sampler=sampler), seed=23)
        nxt = res.paths[:, 1].cpu().numpy()
        assert _chisq([(nxt == x).sum() for x in nb], p * nxt.size) > P_MIN
    finally:
        g.close()


@pytest.mark.gpu
def test_node2vec_second_order_gpu(graph):
    from tests.gpu_util import need_gpu
    torch, E = need_gpu()
    g = E.Graph(graph["row"], graph["adj"], graph["weight"], graph["label"])
    try:
        u = _hub(graph, rank=40)
        pairs, probs = _node2vec_pairs(graph, u, 2.0, 0.5)
        res = E.compute(g, np.full(600_000, u, dtype=np.int32), E.Node2Vec(3, 2.0, 0.5), seed=29)
        paths = res.paths.cpu().numpy()
        assert _chisq(_pair_counts(paths, pairs), probs * paths.shape[0]) > P_MIN
    finally:
        g.close()


@pytest.mark.gpu
def test_ppr_visit_law_gpu(graph):
    """PPR batch: every query's visits sum to its steps; lengths are geometric."""
    from tests.gpu_util import need_gpu
    torch, E = need_gpu()
    g = E.Graph(graph["row"], graph["adj"])
    try:
        src = G.all_sources(torch.from_numpy(graph["row"]), seed=2).numpy()
        src = np.resize(src, 200_000).astype(np.int32)
        res = E.compute(g, src, E.PPR(0.2), seed=41, record_paths=False)
        moves = res.lengths.cpu().numpy() - 1
        k = np.arange(1, 30)
        expected = 0.8 ** (k - 1) * 0.2
        obs = np.array([(moves == x).sum() for x in k])
        assert _chisq(np.append(obs, (moves >= 30).sum()), np.append(expected, 0.8 ** 29) * moves.size) > P_MIN
        assert res.steps == int(moves.sum())
    finally:
        g.close()
