"""Dataset tooling (thunderrw_gb300/toolset.py) against the reference's own
EdgeList2CSR output (tests/golden/make_toolset_golden.py)."""
import os

import numpy as np

from thunderrw_gb300 import formats, toolset

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_edgelist_to_csr_matches_reference_tool(tmp_path):
    assert toolset.main(["EdgeList2CSR", os.path.join(GOLDEN, "edgelist"), str(tmp_path), "#"]) == 0
    for name in ("b_degree.bin", "b_adj.bin"):
        with open(os.path.join(GOLDEN, "edgelist_csr", name), "rb") as f:
            want = f.read()
        with open(os.path.join(str(tmp_path), name), "rb") as f:
            assert f.read() == want, name
    g = formats.load_csr(str(tmp_path))
    row, adj = g["row"], g["adj"]
    assert np.diff(row)[7] == 0  # isolated id inside the range
    for v in range(g["n"]):
        nb = adj[row[v]:row[v + 1]]
        assert np.all(np.diff(nb) > 0) and not np.any(nb == v)  # sorted, simple


def test_edges_to_csr_is_the_symmetric_simple_graph():
    pairs = np.array([[3, 1], [1, 3], [2, 2], [0, 4], [4, 0], [1, 0]])
    row, adj = toolset.edges_to_csr(np.sort(pairs, axis=1))
    assert row.tolist() == [0, 2, 4, 4, 5, 6]
    assert adj.tolist() == [1, 4, 0, 3, 1, 0]


def test_assign_weight_and_label(tmp_path):
    toolset.main(["EdgeList2CSR", os.path.join(GOLDEN, "edgelist"), str(tmp_path)])
    w = toolset.assign_weight(str(tmp_path), 1.0, 5.0, seed=3)
    lab = toolset.assign_edge_label(str(tmp_path), 5, seed=4)
    g = formats.load_csr(str(tmp_path), edge_weight=True, edge_label=True)
    assert np.array_equal(g["weight"], w) and np.array_equal(g["label"], lab)
    assert w.size == g["e"] and w.min() >= 1.0 and w.max() < 5.0
    assert lab.min() >= 0 and lab.max() <= 4
    assert np.array_equal(toolset.assign_weight(str(tmp_path), 1.0, 5.0, seed=3), w)  # seeded


def test_usage():
    assert toolset.main([]) == 2
    assert toolset.main(["AssignWeight", "x"]) == 2
