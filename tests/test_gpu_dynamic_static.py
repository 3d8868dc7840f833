"""Dynamic mode with walker-independent weights (DeepWalk, GenericWalk, PPR)
runs on the static tables: its per-step prefix / alias table / row maximum
would be the static one.  Alias and rejection keep the per-step form on
graphs with a row without positive weight (there dynamic and static differ);
every case equals the oracle's dynamic walk."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu


def _graph(kind):
    from thunderrw_gb300 import generators as G
    g = G.make_graph("chunglu", 1 << 12, 12, seed=71)
    row, adj, w = g["row"].numpy(), g["adj"].numpy(), g["weight"].numpy().copy()
    deg = np.diff(row)
    if kind == "zero_rows":  # every 7th non-empty row weighs nothing
        for v in np.nonzero(deg)[0][::7]:
            w[row[v]:row[v + 1]] = 0.0
    elif kind == "zero_entries":  # zeros inside rows that keep a positive weight
        w[::5] = 0.0
        for v in np.nonzero(deg)[0]:
            if not (w[row[v]:row[v + 1]] > 0).any():
                w[row[v]] = 0.5
    return row, adj, w


@pytest.mark.parametrize("kind", ["positive", "zero_entries", "zero_rows"])
@pytest.mark.parametrize("sampler", ["its", "alias", "rejection"])
def test_dynamic_walker_independent_matches_oracle(kind, sampler):
    torch, E = need_gpu()
    row, adj, w = _graph(kind)
    src = np.nonzero(np.diff(row))[0].astype(np.int32)
    og = O.Graph(row, adj, w)
    d = O.make_desc("deepwalk", "dynamic", sampler, length=12, seed=33)
    ref = O.walk(og, d, src, path_cap=12)
    g = E.Graph(row, adj, w)
    try:
        r = E.compute(g, src, E.DeepWalk(12, mode="dynamic", sampler=sampler), seed=33)
        np.testing.assert_array_equal(r.paths.cpu().numpy(), ref["paths"])
        np.testing.assert_array_equal(r.lengths.cpu().numpy(), ref["lengths"])
        assert r.steps == ref["steps"]
        if kind == "zero_rows" and sampler != "its":
            assert (r.lengths.cpu().numpy() < 12).any()  # walkers stop on the weightless rows
        # PPR (unit weights) in dynamic mode as well
        dq = O.make_desc("ppr", "dynamic", sampler, length=1, tp=0.25, seed=34)
        refq = O.walk(og, dq, src[:40], per_query=50, want_counts=True, want_lengths=False)
        counts, steps = E.ppr_batch(g, src[:40], 50, tp=0.25, seed=34, mode="dynamic", sampler=sampler)
        np.testing.assert_array_equal(counts.cpu().numpy(), refq["counts"])
    finally:
        g.close()
