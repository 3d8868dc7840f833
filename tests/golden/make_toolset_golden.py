"""Generates the EdgeList2CSR fixture: a seeded text edge list with comment
lines, repeated edges in both orientations and self loops
(tests/golden/edgelist/b_edge_list.bin), converted by the reference's own
EdgeList2CSR tool (oracle/_ref/edgelist_to_csr, built by oracle/build_oracle.py
from the reference tree) into tests/golden/edgelist_csr/b_degree.bin and
b_adj.bin.  Run from the repository root where the reference tree exists."""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
IN_DIR = os.path.join(ROOT, "tests", "golden", "edgelist")
OUT_DIR = os.path.join(ROOT, "tests", "golden", "edgelist_csr")


def main():
    tool = os.path.join(ROOT, "oracle", "_ref", "edgelist_to_csr")
    if not os.path.exists(tool):
        sys.exit("build the reference tool first: python oracle/build_oracle.py")
    rng = np.random.default_rng(2024)
    n = 300
    e = rng.integers(0, n, size=(1500, 2))
    e[:40, 1] = e[:40, 0]                      # self loops
    e = np.concatenate([e, e[100:300], e[300:400, ::-1]])  # repeats, both orientations
    e = e[rng.permutation(len(e))]
    e[e == 7] = 299                            # vertex 7 stays isolated inside the id range
    os.makedirs(IN_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    with open(os.path.join(IN_DIR, "b_edge_list.bin"), "w") as f:
        f.write("# seeded test edge list\n")
        for i, (a, b) in enumerate(e):
            if i % 250 == 0:
                f.write("# comment %d\n" % i)
            f.write("%d %d\n" % (a, b))
    subprocess.run([tool, IN_DIR, OUT_DIR, "#"], check=True, stdout=subprocess.DEVNULL)
    print("wrote", sorted(os.listdir(OUT_DIR)))


if __name__ == "__main__":
    main()
