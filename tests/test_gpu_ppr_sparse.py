"""Sparse per-query PPR counts (trw_ppr_batch_sparse) against the dense
counts of the oracle and of trw_ppr_batch, and determinism of the output
order across engines (different schedules)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import need_gpu
from tests.sparse_order import canonical as _canonical, table_bits as _table_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat():
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 13, 16, seed=21)
    return {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in g.items()}


def _check_against_dense(sp, dense):
    off = sp.offsets.cpu().numpy()
    vert = sp.vertices.cpu().numpy()
    cnt = sp.counts.cpu().numpy()
    Q = off.size - 1
    for q in range(Q):
        v, c = vert[off[q]:off[q + 1]], cnt[off[q]:off[q + 1]]
        nz = np.nonzero(dense[q])[0]
        assert v.size == nz.size, q
        assert np.all(c > 0)
        order = np.argsort(v)
        np.testing.assert_array_equal(v[order], nz)
        np.testing.assert_array_equal(c[order], dense[q][nz])


def _check_canonical(sp, bits):
    off = sp.offsets.cpu().numpy()
    vert = sp.vertices.cpu().numpy()
    for q in range(off.size - 1):
        v = vert[off[q]:off[q + 1]]
        np.testing.assert_array_equal(v, _canonical(v, bits), err_msg=f"query {q}")


def test_sparse_matches_oracle_and_dense(rmat):
    torch, E = need_gpu()
    from thunderrw_gb300 import generators as G
    qs = G.random_sources(torch.from_numpy(rmat["row"]), 41, seed=3).numpy()
    og = O.Graph(rmat["row"], rmat["adj"])
    ref = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=77), qs, per_query=700,
                 want_counts=True, want_lengths=False)
    g = E.Graph(rmat["row"], rmat["adj"])
    try:
        outs = []
        for engine in ("persistent", "plain"):
            sp = E.ppr_batch_sparse(g, qs, 700, tp=0.2, seed=77, engine=engine)
            assert sp.steps == ref["steps"]
            _check_against_dense(sp, ref["counts"])
            outs.append(sp)
        total = int(outs[0].offsets[-1].item())
        # the order inside each query is canonical: identical under both schedules
        assert torch.equal(outs[0].offsets, outs[1].offsets)
        assert torch.equal(outs[0].vertices[:total], outs[1].vertices[:total])
        assert torch.equal(outs[0].counts[:total], outs[1].counts[:total])
        _check_canonical(outs[0], _table_bits(700, 0.2, g.n))
        dense, _ = E.ppr_batch(g, qs, 700, tp=0.2, seed=77)
        _check_against_dense(outs[0], dense.cpu().numpy())
        assert torch.equal(outs[0].dense(g.n), dense)
    finally:
        g.close()


def test_sparse_capacity_and_reuse(rmat):
    """Too small a capacity reports the size needed; the tables are left clean."""
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G
    qs = G.random_sources(torch.from_numpy(rmat["row"]), 9, seed=4)
    g = E.Graph(rmat["row"], rmat["adj"])
    try:
        good = E.ppr_batch_sparse(g, qs, 300, tp=0.25, seed=5)
        need = int(good.offsets[-1].item())
        L = N.load()
        off = np.zeros(10, dtype=np.int64)
        v = np.zeros(8, dtype=np.int32)
        c = np.zeros(8, dtype=np.int32)
        steps = np.zeros(1, dtype=np.uint64)
        d = E.PPR(0.25).desc(5)
        src = qs.numpy().astype(np.int32)
        rc = L.trw_ppr_batch_sparse(g.handle, ctypes.byref(d), src.ctypes.data, 9, 300, off.ctypes.data,
                                    v.ctypes.data, c.ctypes.data, 8, steps.ctypes.data, 0, None)
        assert rc == -7 and off[-1] == need
        again = E.ppr_batch_sparse(g, qs, 300, tp=0.25, seed=5)
        assert torch.equal(again.offsets, good.offsets)
        assert torch.equal(again.vertices[:need], good.vertices[:need])
        assert torch.equal(again.counts[:need], good.counts[:need])
        # host buffers of the right size through the raw C ABI
        v = np.zeros(need, dtype=np.int32)
        c = np.zeros(need, dtype=np.int32)
        rc = L.trw_ppr_batch_sparse(g.handle, ctypes.byref(d), src.ctypes.data, 9, 300, off.ctypes.data,
                                    v.ctypes.data, c.ctypes.data, need, steps.ctypes.data, 0, None)
        assert rc == 0 and int(steps[0]) == good.steps
        np.testing.assert_array_equal(v, good.vertices[:need].cpu().numpy())
        np.testing.assert_array_equal(c, good.counts[:need].cpu().numpy())
    finally:
        g.close()


@pytest.mark.parametrize("pinned", [False, True])
def test_sparse_host_ranges_match_device(rmat, pinned):
    """With host outputs a large batch runs as several query ranges whose
    copies overlap the next range's walk; the result equals the one-range
    device-output batch entry for entry, and the oracle for sampled queries."""
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G
    Q, wpq = 61, 160_000  # ~9.8 M walkers: 3 ranges of 21, 21, 19 queries on 152 SMs (8 walkers per lane each)
    qs = G.random_sources(torch.from_numpy(rmat["row"]), Q, seed=8)
    g = E.Graph(rmat["row"], rmat["adj"])
    try:
        dev = E.ppr_batch_sparse(g, qs, wpq, tp=0.2, seed=31)
        need = int(dev.offsets[-1].item())
        L = N.load()

        def host(n, dtype):
            t = torch.zeros(n, dtype=dtype)
            return t.pin_memory() if pinned else t
        off, v, c, steps = host(Q + 1, torch.int64), host(need, torch.int32), host(need, torch.int32), host(1, torch.int64)
        src = qs.to(torch.int32).contiguous()
        src = src.pin_memory() if pinned else src
        d = E.PPR(0.2).desc(31)
        rc = L.trw_ppr_batch_sparse(g.handle, ctypes.byref(d), src.data_ptr(), Q, wpq, off.data_ptr(), v.data_ptr(),
                                    c.data_ptr(), need, steps.data_ptr(), 0, None)
        assert rc == 0, L.trw_last_error()
        assert int(steps[0]) == dev.steps
        assert torch.equal(off, dev.offsets.cpu())
        assert torch.equal(v, dev.vertices[:need].cpu())
        assert torch.equal(c, dev.counts[:need].cpu())
        og = O.Graph(rmat["row"], rmat["adj"])
        for q in (0, 30, 60):  # first range, the middle range, the last (shorter) range
            ref = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=31),
                         qs.numpy()[q:q + 1], per_query=wpq, id_base=q * wpq, want_counts=True, want_lengths=False)
            lo, hi = int(off[q]), int(off[q + 1])
            dense = np.zeros(g.n, dtype=np.int32)
            dense[v[lo:hi].numpy()] = c[lo:hi].numpy()
            np.testing.assert_array_equal(dense, ref["counts"][0])
    finally:
        g.close()


@pytest.mark.parametrize("n", [512, 1024, 4096])
def test_sparse_order_with_wrapping_runs(n):
    """Dense visits (every query reaches most of the graph) fill tables of
    2n slots to about half, so long runs and runs that wrap around the table
    end are common; the output order must be the canonical one under both
    schedules, and the counts the oracle's.  Tables of 1024 slots take the
    32-slots-a-warp emit kernel, larger ones the 128-slots-a-warp one."""
    torch, E = need_gpu()
    from thunderrw_gb300 import generators as G
    g = G.make_graph("er", n, 48, seed=5, weights=False)
    row, adj = g["row"].numpy(), g["adj"].numpy()
    qs = G.random_sources(g["row"], 96, seed=6).numpy()
    og = O.Graph(row, adj)
    ref = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=9), qs, per_query=4000,
                 want_counts=True, want_lengths=False)
    gr = E.Graph(row, adj)
    try:
        a = E.ppr_batch_sparse(gr, qs, 4000, tp=0.2, seed=9, engine="persistent")
        b = E.ppr_batch_sparse(gr, qs, 4000, tp=0.2, seed=9, engine="plain")
        _check_against_dense(a, ref["counts"])
        total = int(a.offsets[-1].item())
        bits = _table_bits(4000, 0.2, n)
        if n == 512:
            assert bits == 10 and total > 96 * 256  # about half of each 1024-slot table is occupied
        _check_canonical(a, bits)
        assert torch.equal(a.offsets, b.offsets)
        assert torch.equal(a.vertices[:total], b.vertices[:total])
        assert torch.equal(a.counts[:total], b.counts[:total])
    finally:
        gr.close()


@pytest.mark.parametrize("queries,wpq", [(1, 40_000), (3, 30_000)])
def test_sparse_large_tables_split_over_ctas(queries, wpq):
    """A query with many walkers gets a table of more than 2^16 slots, which
    the post-processing splits over several CTAs: counts equal the oracle's
    and the order is the same under both schedules."""
    torch, E = need_gpu()
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 17, 8, seed=23, weights=False)
    row, adj = g["row"].numpy(), g["adj"].numpy()
    qs = G.random_sources(g["row"], queries, seed=9).numpy()
    og = O.Graph(row, adj)
    ref = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=19), qs, per_query=wpq,
                 want_counts=True, want_lengths=False)
    gr = E.Graph(row, adj)
    try:
        a = E.ppr_batch_sparse(gr, qs, wpq, tp=0.2, seed=19, engine="persistent")
        b = E.ppr_batch_sparse(gr, qs, wpq, tp=0.2, seed=19, engine="plain")
        _check_against_dense(a, ref["counts"])
        total = int(a.offsets[-1].item())
        bits = _table_bits(wpq, 0.2, 1 << 17)
        assert bits > 16
        _check_canonical(a, bits)
        assert torch.equal(a.offsets, b.offsets)
        assert torch.equal(a.vertices[:total], b.vertices[:total])
        assert torch.equal(a.counts[:total], b.counts[:total])
        again = E.ppr_batch_sparse(gr, qs, wpq, tp=0.2, seed=19)  # the tables were left clean
        assert torch.equal(again.vertices[:total], a.vertices[:total])
    finally:
        gr.close()


def test_sparse_host_weighted_ranges(rmat):
    """A batch of at least 16 units of 8 walkers per lane (and 32 queries)
    runs as 10 query ranges weighted 1,1,2,2,2,2,2,2,1,1 (half-size first and
    last ranges); the result equals the one-range device-output batch and the
    oracle for queries of a small first range, a middle range and the small
    last range."""
    torch, E = need_gpu()
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import generators as G
    Q, wpq = 40, 1_000_000  # 40 M walkers >= 16 x 8 walkers per lane of 152 SMs
    qs = G.random_sources(torch.from_numpy(rmat["row"]), Q, seed=12)
    g = E.Graph(rmat["row"], rmat["adj"])
    try:
        dev = E.ppr_batch_sparse(g, qs, wpq, tp=0.2, seed=51)
        need = int(dev.offsets[-1].item())
        L = N.load()
        off = torch.zeros(Q + 1, dtype=torch.int64).pin_memory()
        v = torch.zeros(need, dtype=torch.int32).pin_memory()
        c = torch.zeros(need, dtype=torch.int32).pin_memory()
        steps = torch.zeros(1, dtype=torch.int64).pin_memory()
        src = qs.to(torch.int32).contiguous().pin_memory()
        d = E.PPR(0.2).desc(51)
        rc = L.trw_ppr_batch_sparse(g.handle, ctypes.byref(d), src.data_ptr(), Q, wpq, off.data_ptr(), v.data_ptr(),
                                    c.data_ptr(), need, steps.data_ptr(), 0, None)
        assert rc == 0, L.trw_last_error()
        assert int(steps[0]) == dev.steps
        assert torch.equal(off, dev.offsets.cpu())
        assert torch.equal(v, dev.vertices[:need].cpu())
        assert torch.equal(c, dev.counts[:need].cpu())
        og = O.Graph(rmat["row"], rmat["adj"])
        for q in (1, 20, 39):  # ranges [0, 2), [20, 25) and [37, 40) of 40 queries
            ref = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=51),
                         qs.numpy()[q:q + 1], per_query=wpq, id_base=q * wpq, want_counts=True, want_lengths=False)
            lo, hi = int(off[q]), int(off[q + 1])
            dense = np.zeros(g.n, dtype=np.int32)
            dense[v[lo:hi].numpy()] = c[lo:hi].numpy()
            np.testing.assert_array_equal(dense, ref["counts"][0])
    finally:
        g.close()
