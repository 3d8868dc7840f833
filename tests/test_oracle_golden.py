"""The oracle restatement (oracle/trw_oracle.cpp) against the golden fixtures
produced by the reference's own sampler code: bit-exact paths, lengths, visit
counts, step counts and static tables."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden_cases import CASES, PHILOX_KAT, case_arrays, case_id, graph_arrays


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_known_answers(ctr, key, out):
    assert list(O.philox(ctr, key)) == out


def _oracle_graph(case):
    ga = graph_arrays(case["graph"])
    return O.Graph(ga["row"], ga["adj"], ga["weight"], ga["label"])


def _desc(case):
    return O.make_desc(case["app"], case["mode"], case["sampler"], length=case["length"], p=case["p"],
                       q=case["q"], tp=case["tp"], schema=case["schema"], seed=case["seed"])


@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_oracle_matches_reference(case):
    g = _oracle_graph(case)
    ref = case_arrays(case)
    if case["mode"] == "static":
        g.build_tables(case["sampler"], 1 if case["app"] == "ppr" else 0)
        if case["sampler"] == "alias":
            assert g.alias.tobytes() == ref["alias"].tobytes()
        elif case["sampler"] == "its":
            assert g.prefix.tobytes() == ref["prefix"].tobytes()
        else:
            assert g.rej_weight.tobytes() == ref["rejw"].tobytes()
            assert g.rej_max.tobytes() == ref["rejmax"].tobytes()
    out = O.walk(g, _desc(case), ref["sources"], per_query=case["per_query"], id_base=case["id_base"],
                 path_cap=case["path_cap"], want_counts=True)
    assert out["steps"] == case["steps"]
    np.testing.assert_array_equal(out["lengths"], ref["lengths"])
    np.testing.assert_array_equal(out["paths"], ref["paths"])
    np.testing.assert_array_equal(out["counts"], ref["counts"])


@pytest.mark.parametrize("case", [c for c in CASES if (c["mode"], c["sampler"]) in
                                  (("uniform", "uniform"), ("static", "alias"), ("dynamic", "maxweight_rejection"),
                                   ("dynamic", "its"))], ids=case_id)
def test_interleaved_ring_matches(case):
    """The step-interleaved oracle (timed CPU baseline) walks identically,
    dynamic max-weight rejection and dynamic ITS included."""
    g = _oracle_graph(case)
    if case["mode"] == "static":
        g.build_tables("alias", 1 if case["app"] == "ppr" else 0)
    ref = case_arrays(case)
    out = O.walk(g, _desc(case), ref["sources"], per_query=case["per_query"], id_base=case["id_base"],
                 path_cap=case["path_cap"], want_counts=True, interleaved=True, ring=8, threads=2)
    assert out["steps"] == case["steps"]
    np.testing.assert_array_equal(out["paths"], ref["paths"])
    np.testing.assert_array_equal(out["lengths"], ref["lengths"])
    np.testing.assert_array_equal(out["counts"], ref["counts"])


def test_draws_are_keyed_by_walker_and_step():
    a = O.draw_u32(1, 5, 3, 0)
    assert a == O.draw_u32(1, 5, 3, 0)
    assert a != O.draw_u32(1, 6, 3, 0)
    assert a != O.draw_u32(1, 5, 4, 0)
    assert a != O.draw_u32(2, 5, 3, 0)
    assert O.draw_u32(1, 5, 3, 4) == O.philox([1, 3, 5, 0], [1, 0])[0]
