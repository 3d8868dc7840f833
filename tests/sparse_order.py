"""The canonical output order of the sparse PPR tables, restated on the host
for the GPU tests (test code only)."""
import numpy as np


def table_bits(wpq, tp, n):
    """Table size of a query: 2^bits >= 1.25 x its expected visits, at most 2 n."""
    bits = 10
    while bits < 30 and (1 << bits) < 1.25 * wpq / tp:
        bits += 1
    while bits > 10 and (1 << (bits - 1)) >= 2 * n:
        bits -= 1
    return bits


def canonical(vertices, bits):
    """The emit order of one query's table: linear probing on key v + 1 at
    slot (v * 0x9E3779B1 mod 2^32) >> (32 - bits), whose set of occupied
    slots does not depend on the insertion order; runs of occupied slots in
    slot order with their keys sorted, the run wrapping around the end last."""
    C = 1 << bits
    keys = np.zeros(C, dtype=np.int64)
    for v in np.sort(vertices):
        h = ((int(v) * 0x9E3779B1) & 0xFFFFFFFF) >> (32 - bits)
        while keys[h]:
            h = (h + 1) & (C - 1)
        keys[h] = int(v) + 1
    occ = keys != 0
    head = tail = 0
    if occ[0] and occ[-1]:
        head = int(np.argmin(occ))
        tail = int(np.argmin(occ[::-1]))
    out, run = [], []
    for i in range(head, C - tail):
        if occ[i]:
            run.append(keys[i])
        elif run:
            out += sorted(run)
            run = []
    out += sorted(run)
    out += sorted(list(keys[C - tail:]) + list(keys[:head]))
    return np.array(out, dtype=np.int64) - 1
