"""The stock reference's speed beside the oracle port's (measurement recipe,
test infrastructure only).

Builds the reference's own app programs unmodified -- the real SFMT
generator, step interleaving with its 64-slot ring (types.h:17-21), the
compile definitions and optimisation flags of its CMakeLists.txt -- from the
sources where they lie in the reference tree, into ``oracle/_ref/stock_<app>``
(git-ignored), and times them against the step-interleaved C++ port that the
bench uses as its CPU baseline, on the same graph, the same walkers and the
same host threads.  The reference's sources stay where they are; its x86
intrinsics (``_mm_prefetch``, SSE2 SFMT) keep the binaries on x86 hosts, so
this runs where the reference tree is, not on the GPU hosts.

    python -m oracle.stock_reference [--threads T] [--reference DIR]

prints one JSON line per workload:
  * PPR (creeper.h:336 uniform_compute): the reference's ppr app, W walkers
    from its single source (generate_single_source: the highest-degree vertex,
    walker_generator.cpp:42-57), tp = 0.2, on the R-MAT 2^22 graph of the
    PPR batch benchmark; its own "Throughput (steps per second)" line
    (creeper.h:803);
  * DeepWalk (creeper.h:420 static_compute): the reference's deepwalk app,
    static alias sampling, one walker per vertex, L = 80, on the Chung-Lu 2^18
    graph of the DeepWalk benchmark with its edge weights (-ew).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STOCK_APPS = ["ppr", "deepwalk"]


def _reference_root(arg=None):
    from oracle.build_oracle import reference_root_default
    return arg or reference_root_default()


def build(reference_root=None):
    """g++ over the reference's own files with its own definitions and flags
    (CMakeLists.txt: -std=c++11 -O3 -fopenmp -march=native, USE_LOG,
    TIME_RESULTS; random_walk/CMakeLists.txt: SFMT_MEXP=19937, HAVE_SSE2)."""
    root = _reference_root(reference_root)
    sfmt = os.path.join(root, "dependency", "SFMT-src-1.5.1")
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    defs = ["-DUSE_LOG", "-DTIME_RESULTS", "-DSFMT_MEXP=19937", "-DHAVE_SSE2=1"]
    flags = ["-O3", "-fopenmp", "-march=native", "-w"]
    sfmt_obj = os.path.join(out_dir, "stock_sfmt.o")
    subprocess.check_call(["gcc", *flags, *defs, "-I", sfmt, "-c", os.path.join(sfmt, "SFMT.c"), "-o", sfmt_obj])
    procs = []
    for app in STOCK_APPS:
        # (-include cstdint: the sources use uint32_t without it, which newer
        # libstdc++ headers no longer pull in; random_walk/ holds the
        # headers the apps include by bare name)
        cmd = ["g++", "-std=c++11", *flags, *defs, "-include", "cstdint", "-I", root,
               "-I", os.path.join(root, "random_walk"), "-I", sfmt,
               os.path.join(root, "random_walk", "apps", app + ".cpp"),
               os.path.join(root, "random_walk", "walker_generator.cpp"),
               os.path.join(root, "util", "graph", "graph.cpp"),
               os.path.join(root, "util", "log", "log.cpp"),
               os.path.join(root, "util", "io", "io.cpp"),
               sfmt_obj, "-o", os.path.join(out_dir, "stock_" + app), "-pthread"]
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("stock build failed: " + " ".join(cmd))


def _throughput(out: str) -> float:
    m = re.search(r"Throughput \(steps per second\): ([0-9.eE+]+)", out)
    if not m:
        raise RuntimeError("no throughput line in the reference's output:\n" + out[-2000:])
    return float(m.group(1))


def _run_stock(app, graph_dir, args, threads):
    exe = os.path.join(HERE, "_ref", "stock_" + app)
    cmd = [exe, "-f", graph_dir + os.sep, "-n", str(threads), *args]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s failed (%d):\n%s" % (" ".join(cmd), r.returncode, r.stdout[-2000:]))
    return _throughput(r.stdout)


def _graph(kind, n, deg):
    """The benchmark's graph (bench.py's generator and seed), on the host."""
    sys.path.insert(0, ROOT)
    from thunderrw_gb300 import generators as G
    g = G.make_graph(kind, n, deg, seed=20240601, device="cpu", weights=kind != "rmat")
    w = g.get("weight")
    return g["row"].numpy(), g["adj"].numpy(), (w.numpy() if w is not None else None)


def time_ppr(threads, walkers, reps=3):
    from oracle import oracle as O
    from thunderrw_gb300 import formats
    row, adj, _ = _graph("rmat", 1 << 22, 32)
    deg = row[1:] - row[:-1]
    src = int(deg.argmax())  # generate_single_source's vertex (the first of the highest degree)
    with tempfile.TemporaryDirectory() as d:
        formats.store_csr(d, row, adj)
        stock = [_run_stock("ppr", d, ["-sp", "0.2", "-nw", str(walkers)], threads) for _ in range(reps)]
    og = O.Graph(row, adj)
    desc = O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2, seed=7)
    port = []
    for i in range(reps):
        t0 = time.perf_counter()
        r = O.walk(og, desc, [src], per_query=walkers, id_base=i * walkers, want_lengths=False, num_queries=1,
                   threads=threads, interleaved=True, ring=64)
        port.append(r["steps"] / (time.perf_counter() - t0))
    return {"workload": "ppr single source (highest degree) tp=0.2, rmat 2^22 deg 32", "walkers": walkers,
            "threads": threads, "stock_steps_per_s": max(stock), "port_steps_per_s": max(port),
            "port_over_stock": max(port) / max(stock)}


def time_deepwalk(threads, reps=3):
    from oracle import oracle as O
    from thunderrw_gb300 import formats
    row, adj, w = _graph("chunglu", 1 << 18, 16)
    with tempfile.TemporaryDirectory() as d:
        formats.store_csr(d, row, adj, weight=w)
        # -ew: edge weights (the app's weight() reads them); -em 1: static
        # execution, -sm 2: alias sampling (types.h), -l 80
        stock = [_run_stock("deepwalk", d, ["-ew", "-em", "1", "-sm", "2", "-l", "80"], threads)
                 for _ in range(reps)]
    og = O.Graph(row, adj, w)
    og.build_tables("alias", 0)
    desc = O.make_desc("deepwalk", "static", "alias", length=80, seed=11)
    import numpy as np
    src = np.arange(row.size - 1, dtype=np.int32)
    port = []
    for i in range(reps):
        t0 = time.perf_counter()
        r = O.walk(og, desc, src, id_base=i * src.size, path_cap=80, threads=threads, interleaved=True, ring=64)
        port.append(r["steps"] / (time.perf_counter() - t0))
    return {"workload": "deepwalk static alias, chung-lu 2^18 deg 16, one walker per vertex, L=80",
            "threads": threads, "stock_steps_per_s": max(stock), "port_steps_per_s": max(port),
            "port_over_stock": max(port) / max(stock)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--walkers", type=int, default=4_000_000)
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    build(a.reference)
    print(json.dumps(time_ppr(a.threads, a.walkers)), flush=True)
    print(json.dumps(time_deepwalk(a.threads)), flush=True)


if __name__ == "__main__":
    main()
