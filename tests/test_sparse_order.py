"""The host restatement of the sparse PPR output order (tests/sparse_order.py),
checked on the CPU: the GPU tests compare the emit kernel's per-query order
with it, so it must hold for any insertion order the walk's atomics produce."""
import numpy as np
import pytest

from tests.sparse_order import canonical, table_bits


def _home(v, bits):
    return ((int(v) * 0x9E3779B1) & 0xFFFFFFFF) >> (32 - bits)


def _insert(order, bits):
    """Linear probing on key v + 1 in the given insertion order (as the walk's
    CAS inserts do, one at a time)."""
    C = 1 << bits
    keys = np.zeros(C, dtype=np.int64)
    for v in order:
        h = _home(v, bits)
        while keys[h]:
            h = (h + 1) & (C - 1)
        keys[h] = int(v) + 1
    return keys


def _runs_in_slot_order(keys):
    """Runs of occupied slots in slot order, keys sorted inside a run, the run
    wrapping around the table end last."""
    C = keys.size
    occ = keys != 0
    # Walk the cycle from the first empty slot when a run crosses slot
    # C-1 -> 0: that run is then collected last, and the others in slot order.
    start = int(np.argmin(occ)) if occ[0] and occ[-1] and not occ.all() else 0
    out, run = [], []
    for j in range(C):
        i = (start + j) % C
        if occ[i]:
            run.append(int(keys[i]))
        elif run:
            out += sorted(run)
            run = []
    out += sorted(run)
    return np.array(out, dtype=np.int64) - 1


@pytest.mark.parametrize("bits,n,seed", [(10, 300, 1), (10, 700, 2), (12, 2500, 3), (11, 1300, 4)])
def test_any_insertion_order_gives_the_canonical_order(bits, n, seed):
    rng = np.random.default_rng(seed)
    verts = rng.choice(1 << 20, n, replace=False)
    want = canonical(verts, bits)
    assert sorted(want.tolist()) == sorted(verts.tolist())
    occupied = None
    for _ in range(4):
        keys = _insert(rng.permutation(verts), bits)
        if occupied is None:
            occupied = keys != 0
        # the set of occupied slots does not depend on the insertion order
        np.testing.assert_array_equal(keys != 0, occupied)
        np.testing.assert_array_equal(_runs_in_slot_order(keys), want)


def test_wrapping_run_comes_last():
    bits = 10
    C = 1 << bits
    at_end = [v for v in range(1 << 16) if _home(v, bits) == C - 1][:3]
    at_mid = [v for v in range(1 << 16) if _home(v, bits) == C // 2][:2]
    verts = np.array(at_end + at_mid)
    out = canonical(verts, bits)
    # the middle run (two keys, sorted) first, then the run through slots C-1, 0, 1
    assert out.tolist() == sorted(at_mid) + sorted(at_end)
    keys = _insert(verts[::-1], bits)
    assert keys[C - 1] and keys[0] and keys[1] and not keys[2]
    np.testing.assert_array_equal(_runs_in_slot_order(keys), out)


def test_table_bits():
    # 10^4 walkers at tp 0.2: 5 x 10^4 expected visits -> 2^16 slots (>= 1.25 x visits)
    assert table_bits(10_000, 0.2, 1 << 22) == 16
    # never above 2 n slots for a small graph
    assert table_bits(10_000, 0.2, 3000) == 13
    # at least 2^10
    assert table_bits(10, 0.5, 1 << 22) == 10
