"""Generates the committed golden fixtures by running the REFERENCE's own
sampler code (oracle/_ref harness binaries, compiled from the ThunderRW tree
with the Philox SFMT.h shim) on small seeded graphs.

Run in a container that holds the reference tree:
    python tests/golden/make_golden.py [/path/to/ThunderRW]

Writes tests/golden/graphs.npz, tests/golden/cases.npz and
tests/golden/manifest.json.  The fixtures are then read by the CPU tests
(oracle restatement vs reference) and the GPU tests (CUDA path vs reference).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle, oracle as O  # noqa: E402
from thunderrw_gb300 import generators as G  # noqa: E402

# Random123 known-answer vectors for Philox4x32-10 (counter, key, output).
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]

GRAPHS = {
    "rmat512": dict(kind="rmat", n=512, avg_degree=10, seed=7, labels=5),
    "chunglu512": dict(kind="chunglu", n=512, avg_degree=8, seed=9, labels=5),
    "er300": dict(kind="er", n=300, avg_degree=3, seed=5, labels=3),
}

SCHEMA = [0, 1, 2, 3, 4]


def cases():
    out = []
    for gname in GRAPHS:
        schema = SCHEMA if gname != "er300" else [0, 1, 2]
        for app, mode, sm in [
            ("deepwalk", "static", "alias"), ("deepwalk", "static", "its"), ("deepwalk", "static", "rejection"),
            ("deepwalk", "dynamic", "its"), ("deepwalk", "dynamic", "alias"), ("deepwalk", "dynamic", "rejection"),
            ("deepwalk", "dynamic", "maxweight_rejection"), ("deepwalk", "uniform", "uniform"),
            ("ppr", "uniform", "uniform"), ("ppr", "static", "alias"),
            ("node2vec", "dynamic", "maxweight_rejection"), ("node2vec", "dynamic", "its"),
            ("metapath", "dynamic", "its"), ("metapath", "dynamic", "alias"), ("metapath", "dynamic", "rejection"),
            ("genericwalk", "static", "its"), ("genericwalk", "static", "alias"), ("genericwalk", "dynamic", "its"),
        ]:
            L = 20 if gname != "chunglu512" else 30
            out.append(dict(graph=gname, app=app, mode=mode, sampler=sm, length=L,
                            path_cap=1 if app == "ppr" else L, seed=11 + len(out), id_base=3 * len(out),
                            p=2.0, q=0.5, tp=0.2, schema=schema if app == "metapath" else None,
                            num_walkers=160, per_query=0))
    # PPR batch: 4 queries x 48 walkers, walker id = q * 48 + j
    out.append(dict(graph="rmat512", app="ppr", mode="uniform", sampler="uniform", length=1, path_cap=1,
                    seed=1, id_base=0, p=1.0, q=1.0, tp=0.2, schema=None, num_walkers=4, per_query=48))
    return out


def main(reference_root=None):
    """reference_root: the reference tree (default: build_oracle's
    TRW_REFERENCE_ROOT / mount rule)."""
    build_oracle.build(reference_root, with_ref=True)
    graphs, arrays, manifest = {}, {}, {"philox_kat": PHILOX_KAT, "graphs": GRAPHS, "cases": []}
    gobjs = {}
    for name, spec in GRAPHS.items():
        spec = dict(spec)
        g = G.make_graph(spec.pop("kind"), spec.pop("n"), spec.pop("avg_degree"), spec.pop("seed"),
                         labels=spec.pop("labels"))
        gobjs[name] = O.Graph(g["row"], g["adj"], g["weight"], g["label"])
        for k in ("row", "adj", "weight", "label"):
            graphs[name + "/" + k] = getattr(gobjs[name], k)
    for i, c in enumerate(cases()):
        gr = gobjs[c["graph"]]
        sources = G.all_sources(__import__("torch").from_numpy(gr.row), seed=100 + i).numpy()
        sources = sources[: c["num_walkers"]]
        key = "c%02d" % i
        if c["per_query"] > 0:
            paths, lengths, counts, steps = [], [], [], 0
            for qi, s in enumerate(sources):
                srcs = np.full(c["per_query"], s, dtype=np.int32)
                r = O.run_reference(gr, c["app"], c["mode"], c["sampler"], srcs, length=c["length"],
                                    path_cap=c["path_cap"], seed=c["seed"], id_base=qi * c["per_query"],
                                    p=c["p"], q=c["q"], tp=c["tp"], schema=c["schema"])
                paths.append(r["paths"]); lengths.append(r["lengths"]); counts.append(r["counts"])
                steps += r["steps"]
            ref = {"paths": np.concatenate(paths), "lengths": np.concatenate(lengths),
                   "counts": np.stack(counts), "steps": steps}
        else:
            ref = O.run_reference(gr, c["app"], c["mode"], c["sampler"], sources, length=c["length"],
                                  path_cap=c["path_cap"], seed=c["seed"], id_base=c["id_base"],
                                  p=c["p"], q=c["q"], tp=c["tp"], schema=c["schema"])
            ref["counts"] = ref["counts"][None, :]
        arrays[key + "/sources"] = sources.astype(np.int32)
        for k in ("paths", "lengths", "counts"):
            arrays[key + "/" + k] = ref[k]
        for k in ("alias", "prefix", "rejw", "rejmax"):
            if k in ref:
                arrays[key + "/" + k] = ref[k]
        c = dict(c, key=key, steps=int(ref["steps"]))
        manifest["cases"].append(c)
        print(key, c["graph"], c["app"], c["mode"], c["sampler"], "steps", c["steps"])
    np.savez_compressed(os.path.join(HERE, "graphs.npz"), **graphs)
    np.savez_compressed(os.path.join(HERE, "cases.npz"), **arrays)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main(*sys.argv[1:2])
