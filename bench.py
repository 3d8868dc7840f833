#!/usr/bin/env python
"""Walk-steps/s benchmark of the GB300 random-walk engine.

Default workload (the batched-PPR configuration): R-MAT graph (a,b,c =
0.57,0.19,0.19), N = 2^22 vertices, average degree 32 before symmetrisation,
undirected int32 CSR; 4096 queries x 10^4 walkers whose sources are drawn
uniformly among non-isolated vertices; uniform sampling, termination
probability 0.2 after every move (geometric lengths, mean 5); output: int32
visit counts per query as sparse CSR (offsets, vertex, count).  One step =
one whole batch through trw_ppr_batch_sparse.  Inputs (adjacency 0.5 GB,
per-query tables 2 GiB) are far larger than the 129 MB L2, so no separate
flush is needed.

After the headline workload the default run measures the other single-GPU
workloads for a few steps each (``workloads`` key): DeepWalk static alias
(Chung-Lu 2^18), Node2Vec max-weight rejection (R-MAT 2^24) and MetaPath
dynamic ITS (R-MAT 2^24).  Every workload's last timed batch is checked
against the CPU oracle on a sample, outside the timed region
(``parity_checked``).

Prints one JSON line (rank 0).  --impl reference times the reference's CPU
algorithm (the step-interleaved C++ oracle port of creeper.h's ring) on the
host cores instead, with the same ``config``.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from types import SimpleNamespace

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from thunderrw_gb300 import bytes_model, replicas  # noqa: E402

BYTES_PER_STEP = {
    # Algorithmic bytes per move (32-byte sectors of each independent random
    # access, 4 bytes per path entry), thunderrw_gb300/bytes_model.py:
    # row pair 32 + adjacency entry 32 + visit-count update 32.
    "ppr": bytes_model.UNIFORM_PPR,
    # row pair 32 + alias slot 32 + path entry 4
    "deepwalk": bytes_model.STATIC_ALIAS,
}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per step of each
# workload's walk kernel, from one ncu capture of that kernel: PPR on the
# full N = 2^22 graph with 256 queries (1.259 GB over 12.80 M steps; the full
# batch's tables do not change the per-step traffic of the walk: only the
# in-flight queries' tables are written), DeepWalk, Node2Vec and MetaPath on
# their full graphs (each in the form the autotuner picks: DeepWalk one
# walker per lane and 4 CTAs per SM, Node2Vec and MetaPath the plain form
# with the 16-byte entries that carry the next step's row or block).
# Scaled by the steps of one full launch.
TRAFFIC_BYTES_PER_STEP = {
    "ppr": 98.34,
    "ppr_dense": 89.13,
    "deepwalk": 14.01,
    "node2vec": 209.88,
    "metapath": 150.24,
}

WORKLOADS = {
    "ppr": dict(kind="rmat", n=1 << 22, deg=32, queries=4096, per_query=10_000, tp=0.2,
                name="ppr_batch rmat(0.57,0.19,0.19) N=2^22 deg=32 undirected, 4096 queries x 1e4 walkers, "
                     "uniform sampling tp=0.2, int32 visit counts per query"),
    "deepwalk": dict(kind="chunglu", n=1 << 18, deg=16, length=80,
                     name="deepwalk static alias chung-lu(2.1) N=2^18 deg=16, one walker per vertex, L=80"),
    "node2vec": dict(kind="rmat", n=1 << 24, deg=16, length=80, p=2.0, q=0.5,
                     name="node2vec p=2 q=0.5 dynamic max-weight rejection rmat N=2^24 deg=16, one walker per "
                          "vertex, L=80"),
    "metapath": dict(kind="rmat", n=1 << 24, deg=32, length=20, walkers=1 << 22, labels=5, schema=[0, 1, 2, 3, 4],
                     name="metapath schema 0..4 dynamic ITS rmat N=2^24 deg=32, 5 labels, 2^22 random sources, L=20"),
}
SIDE_WORKLOADS = ("deepwalk", "node2vec", "metapath")
L2_BYTES = 129e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ppr", choices=sorted(WORKLOADS) + ["serving"])
    ap.add_argument("--rates", default="50,200,800,1600,3200", help="serving: arrival rates (requests/s)")
    ap.add_argument("--inflight", type=int, default=4, help="serving: batches in flight (streams)")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--queries", type=int, default=None, help="override the query count (small runs)")
    ap.add_argument("--scale", type=int, default=None, help="override log2(N) (small runs)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-tune", action="store_true", help="keep the automatic launch shape (no autotuning)")
    ap.add_argument("--no-workloads", action="store_true", help="measure the headline workload only")
    ap.add_argument("--no-parity", action="store_true", help="skip the untimed oracle check of a timed batch")
    ap.add_argument("--side-steps", type=int, default=5, help="timed steps of each side workload")
    ap.add_argument("--shape", default=None, help="walkers_per_lane,ctas_per_sm: set this launch shape, no tuning")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--dense", action="store_true", help="PPR: dense Q x N count output instead of sparse CSR")
    return ap.parse_args()


def dist_env():
    return replicas.rank_env()


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload construction and description (shared by both arms)
# ---------------------------------------------------------------------------

def workload_name(wl, over):
    """The workload's name, with any size override spelled out."""
    extra = []
    if over.scale:
        extra.append("N=2^%d" % over.scale)
    if over.queries:
        extra.append("%d queries" % over.queries)
    return wl["name"] + (" [reduced: %s]" % ", ".join(extra) if extra else "")


def needs_l2_flush(name, n, e):
    """Working sets that fit in the 129 MB L2 are flushed between timed steps."""
    working = e * 4 + n * 8 + (e * 16 if name == "deepwalk" else 0)
    return working < 2 * L2_BYTES


def workload_config(name, wl, over, n, e, walkers):
    """The ``config`` of the JSON line: the same dict in both arms."""
    cfg = {"workload": workload_name(wl, over), "n": int(n), "e": int(e)}
    if "queries" in wl:
        q = over.queries or wl["queries"]
        # every visited vertex has a neighbour (undirected graph, non-isolated
        # sources), so a walker makes 1/tp moves on average
        cfg.update(queries=q, walkers_per_query=wl["per_query"], tp=wl["tp"],
                   steps_per_batch=int(round(q * wl["per_query"] / wl["tp"])))
    else:
        cfg.update(walkers=int(walkers), length=wl["length"])
        if name in ("deepwalk", "node2vec"):  # no dead ends: every walker makes L - 1 moves
            cfg["steps_per_batch"] = int(walkers) * (wl["length"] - 1)
    cfg["l2"] = ("L2 flushed between timed steps (512 MB write outside the events)" if needs_l2_flush(name, n, e)
                 else "inputs larger than L2 (adjacency %.2f GB), no flush" % (e * 4 / 1e9))
    return cfg


def build_inputs(wl, over, device, rank=0):
    """The workload's graph (the same on every rank) and rank's own sources."""
    import torch
    from thunderrw_gb300 import generators as G
    n = 1 << over.scale if over.scale else wl["n"]
    g = G.make_graph(wl["kind"], n, wl["deg"], seed=20240601, device=device,
                     weights=wl["kind"] != "rmat" or "length" in wl, labels=wl.get("labels", 0))
    out = {"n": n, "row": g["row"], "adj": g["adj"], "weight": g["weight"], "label": g["label"]}
    if "queries" in wl:
        q = over.queries or wl["queries"]
        out["sources"] = G.random_sources(g["row"], q, seed=replicas.replica_seed(7, rank) & 0x7FFFFFFF)
        out["per_query"] = wl["per_query"]
    elif "walkers" in wl:
        out["sources"] = G.random_sources(g["row"], wl["walkers"], seed=replicas.replica_seed(7, rank) & 0x7FFFFFFF)
    else:
        out["sources"] = G.all_sources(g["row"], seed=0)
    if torch.device(device).type == "cuda":
        torch.cuda.synchronize()
    return out


def host_arrays(inp):
    def h(k):
        return inp[k].cpu().numpy() if inp.get(k) is not None else None
    return {k: h(k) for k in ("row", "adj", "weight", "label", "sources")}


# ---------------------------------------------------------------------------
# CPU baseline: the step-interleaved port of the reference ring
# ---------------------------------------------------------------------------

def cpu_baseline(name, wl, host, per_query, seconds, threads=0):
    """The step-interleaved CPU port (oracle) on a bounded sample of the same
    workload, on all host threads.  Returns a dict (value, sample, cores, ...).

    PPR: the reference's PPR app counts nothing (ppr.cpp:27-29), so the
    headline value is the count-free walk; the same walks recording visit
    counts into a dense per-query block are timed too (``value_with_counts``),
    with the block zeroed outside the timed passes."""
    from oracle import oracle as O
    og = O.Graph(host["row"], host["adj"], host["weight"], host["label"])
    ncores = threads or os.cpu_count()
    src = np.asarray(host["sources"], dtype=np.int32)
    form = "step-interleaved C++ port of the reference ring (64 walkers per thread)"
    if name == "ppr":
        d = O.make_desc("ppr", "uniform", "uniform", length=1, tp=wl["tp"], seed=11)
        chunk = 64  # queries per pass
        counts = np.zeros((chunk, og.n), dtype=np.int32)
        res = {}
        for with_counts in (False, True):
            total_steps, total_t, done_q = 0, 0.0, 0
            budget = seconds / 2
            while total_t < budget:  # the batch again (fresh walker ids) until the budget is spent
                at = done_q % src.size
                qs = src[at:at + chunk]
                if with_counts:
                    counts[: qs.size].fill(0)  # outside the timed pass
                t0 = time.perf_counter()
                r = O.walk(og, d, qs, per_query=per_query, id_base=done_q * per_query, want_lengths=False,
                           num_queries=qs.size, threads=ncores, interleaved=True, ring=64,
                           out_counts=counts if with_counts else None)
                total_t += time.perf_counter() - t0
                total_steps += r["steps"]
                done_q += qs.size
            res[with_counts] = (total_steps / total_t, done_q, total_steps, total_t)
        v, dq, st, tt = res[False]
        vc, dqc, stc, ttc = res[True]
        sample = ("%s, count-free as the reference's PPR: %d queries x %d walkers (%d steps, %.2f passes over the "
                  "batch) in %.1f s; with dense visit counts (block zeroed outside the timed passes): %d queries, "
                  "%d steps in %.1f s" % (form, dq, per_query, st, dq / src.size, tt, dqc, stc, ttc))
        return {"value": v, "value_with_counts": vc, "sample": sample, "cores": ncores}
    if name == "deepwalk":
        og.build_tables("alias", 0)
        d = O.make_desc("deepwalk", "static", "alias", length=wl["length"], seed=11)
    else:  # dynamic samplers, on the same step-interleaved ring
        d = O.make_desc(name, "dynamic", "maxweight_rejection" if name == "node2vec" else "its",
                        length=wl["length"], p=wl.get("p", 1.0), q=wl.get("q", 1.0), schema=wl.get("schema"), seed=11)
    total_steps, total_t, done = 0, 0.0, 0
    chunk = 1 << 16
    # chunks of the workload's walkers in order; a workload that finishes
    # before the time budget runs again (fresh walker ids) until it is spent
    while total_t < seconds:
        at = done % src.size
        s = src[at:at + chunk]
        t0 = time.perf_counter()
        r = O.walk(og, d, s, id_base=done, path_cap=wl["length"], threads=ncores, interleaved=True, ring=64)
        total_t += time.perf_counter() - t0
        total_steps += r["steps"]
        done += s.size
        del r
    sample = "%s, %d walkers x %d steps (%d steps, %.2f passes over the workload) in %.1f s" % (
        form, done, wl["length"] - 1, total_steps, done / src.size, total_t)
    return {"value": total_steps / total_t, "sample": sample, "cores": ncores}


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------

def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import torch
    wl = WORKLOADS[args.workload]
    have_gpu = torch.cuda.is_available()
    inp = build_inputs(wl, args, "cuda" if have_gpu else "cpu")
    host = host_arrays(inp)
    n, e = inp["n"], int(inp["adj"].numel())
    per_q = inp.get("per_query", 0)
    del inp
    if have_gpu:
        torch.cuda.empty_cache()
    vals, vals_c = [], []
    res = {}
    for i in range(args.warmup + args.steps):
        res = cpu_baseline(args.workload, wl, host, per_q, max(2.0, 20.0 / max(1, args.warmup + args.steps)))
        if i >= args.warmup:
            vals.append(res["value"])
            if "value_with_counts" in res:
                vals_c.append(res["value_with_counts"])
    value = statistics.median(vals)
    cpu = {"value": value, "unit": "steps/s", "cores": res["cores"], "kind": "port",
           "sample": "per step: " + res["sample"]}
    if vals_c:
        cpu["value_with_counts"] = statistics.median(vals_c)
    line = {
        "impl": "reference", "metric": "walk_steps_per_s", "value": value, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic (seeded generator, no dataset)",
        "config": workload_config(args.workload, wl, args, n, e, host["sources"].size),
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def _c(t):
    return ctypes.c_void_p(t.data_ptr())


def parity_sample(name, wl, host, seed, out, per_query):
    """Checks a sample of one timed batch against the CPU oracle, bit for
    bit: the first 8 queries' (vertex, count) lists of a PPR batch, or the
    paths and lengths of the first 2^14 walkers of a walk batch."""
    from oracle import oracle as O
    og = O.Graph(host["row"], host["adj"], host["weight"], host["label"])
    src = host["sources"]
    if name == "ppr":
        nq = min(8, src.size)
        d = O.make_desc("ppr", "uniform", "uniform", length=1, tp=wl["tp"], seed=seed)
        ref = O.walk(og, d, src[:nq], per_query=per_query, want_counts=True, want_lengths=False)
        off, vert, cnt = out
        off = off[: nq + 1].cpu().numpy()
        vert = vert[: off[-1]].cpu().numpy()
        cnt = cnt[: off[-1]].cpu().numpy()
        for q in range(nq):
            v, c = vert[off[q]:off[q + 1]], cnt[off[q]:off[q + 1]]
            nz = np.nonzero(ref["counts"][q])[0]
            order = np.argsort(v)
            if v.size != nz.size or not np.array_equal(v[order], nz) or not np.array_equal(c[order], ref["counts"][q][nz]):
                return False, "query %d differs from the oracle" % q
        return True, "first %d queries' (vertex, count) lists == oracle (%d steps)" % (nq, ref["steps"])
    k = min(src.size, 1 << 14)
    if name == "deepwalk":
        og.build_tables("alias", 0)
        d = O.make_desc("deepwalk", "static", "alias", length=wl["length"], seed=seed)
    else:
        d = O.make_desc(name, "dynamic", "maxweight_rejection" if name == "node2vec" else "its",
                        length=wl["length"], p=wl.get("p", 1.0), q=wl.get("q", 1.0), schema=wl.get("schema"),
                        seed=seed)
    ref = O.walk(og, d, src[:k], path_cap=wl["length"])
    paths, lengths = out
    ok = np.array_equal(paths[:k].cpu().numpy(), ref["paths"]) and np.array_equal(lengths[:k].cpu().numpy(),
                                                                                   ref["lengths"])
    return ok, "first %d walkers' paths and lengths %s oracle (%d steps)" % (k, "==" if ok else "!=", ref["steps"])


def measure(name, args, over, dev, rank, world, steps, warmup, headline):
    """Times one workload through the C ABI; returns its result dict."""
    import torch
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import engine as E

    wl = WORKLOADS[name]
    t_build = time.perf_counter()
    inp = build_inputs(wl, over, dev, rank)
    graph = E.Graph(inp["row"], inp["adj"], inp["weight"], inp.get("label"))
    build_s = time.perf_counter() - t_build
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    L = N.load()
    res = {"config": workload_config(name, wl, over, graph.n, graph.e, inp["sources"].numel()),
           "graph_build_s": build_s}

    sparse = name == "ppr" and not args.dense
    src = inp["sources"]
    steps_dev = torch.zeros(1, dtype=torch.int64, device=dev)
    counts = None
    if name == "ppr":
        Q = src.numel()
        per_q = inp["per_query"]
        if sparse:
            # size the CSR output from one untimed batch (same shape, other seed)
            probe = E.ppr_batch_sparse(graph, src, per_q, tp=wl["tp"], seed=999)
            cap = int(int(probe.offsets[-1].item()) * 1.25) + 1024
            del probe
            offsets = torch.empty(Q + 1, dtype=torch.int64, device=dev)
            vert = torch.empty(cap, dtype=torch.int32, device=dev)
            vcnt = torch.empty(cap, dtype=torch.int32, device=dev)
            outputs = (offsets, vert, vcnt)

            def one_step(seed, engine="persistent"):
                d = E.PPR(wl["tp"]).desc(replicas.replica_seed(seed, rank))
                N.check(L.trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), _c(src), Q, per_q, _c(offsets),
                                               _c(vert), _c(vcnt), cap, _c(steps_dev), N.ENGINES[engine], sp))
            # walk, distinct, segment scan, offsets scan, emit (one query range)
            launches_per_step = 5
        else:
            counts = torch.empty((Q, graph.n), dtype=torch.int32, device=dev)
            outputs = None

            def one_step(seed, engine="persistent"):
                d = E.PPR(wl["tp"]).desc(replicas.replica_seed(seed, rank))
                N.check(L.trw_ppr_batch(graph.handle, ctypes.byref(d), _c(src), Q, per_q, _c(counts),
                                        _c(steps_dev), 1, N.ENGINES[engine], sp))
            launches_per_step = 1
        app = E.PPR(wl["tp"])
    else:
        W = src.numel()
        Lw = wl["length"]
        paths = torch.empty((W, Lw), dtype=torch.int32, device=dev)
        lengths = torch.empty(W, dtype=torch.int32, device=dev)
        outputs = (paths, lengths)
        app = {"deepwalk": E.DeepWalk(Lw),
               "node2vec": E.Node2Vec(Lw, wl.get("p", 2.0), wl.get("q", 0.5)),
               "metapath": E.MetaPath(Lw, wl.get("schema", [0, 1, 2, 3, 4]))}[name]
        if name == "deepwalk":
            graph.build_tables("alias", "edge")

        def one_step(seed, engine="persistent"):
            d = app.desc(replicas.replica_seed(seed, rank))
            N.check(L.trw_walk(graph.handle, ctypes.byref(d), _c(src), W, 0, _c(paths), Lw, _c(lengths), None,
                               _c(steps_dev), N.ENGINES[engine], sp))
        launches_per_step = 1

    # ---- launch shape: tuned once on a sample of this workload, as a user
    # would (thunderrw_gb300/autotune.py), outside every timed region
    shape = "automatic"
    if args.shape and headline:
        slot = "uniform" if name == "ppr" else app.sampler
        r, c = (int(x) for x in args.shape.split(","))
        graph.set_engine_shape(slot, r, c)
        shape = {"slot": slot, "walkers_per_lane": r, "ctas_per_sm": c, "set_by": "--shape"}
    elif not args.no_tune:
        from thunderrw_gb300 import autotune
        if name == "ppr":
            tr = autotune.tune(graph, app, src, walkers_per_query=per_q, rings=(1, 2), ctas=(0, 4), repeats=2)
        else:
            tr = autotune.tune(graph, app, src, rings=(1, 2, 4), ctas=(0, 2, 4), repeats=2)
        shape = {"slot": tr.sampler, "walkers_per_lane": tr.best[0], "ctas_per_sm": tr.best[1],
                 "tuned_on_walkers": tr.walkers, "candidates": len(tr.timings)}
        torch.cuda.synchronize()
    plain_shape = isinstance(shape, dict) and shape["walkers_per_lane"] == -1
    res["engine"] = {"engine": "plain form (the tuned launch shape)" if plain_shape else "persistent",
                     "launch_shape": shape,
                     "output": ("sparse CSR per query (offsets, vertex, int32 count)" if sparse else
                                "dense int32 [Q][N], zeroed every step" if name == "ppr" else
                                "int32 paths [W][L] + lengths")}

    # ---- warm-up
    for i in range(warmup):
        one_step(1000 + i)
    torch.cuda.synchronize()

    # ---- timed region: K whole batches, fresh seeds
    sampler = ClockSampler(dev.index or 0) if headline else None
    if sampler:
        sampler.start()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    flush_l2 = needs_l2_flush(name, graph.n, graph.e)
    flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device=dev) if flush_l2 else None
    if flush_l2:
        t_total = 0.0
        for i in range(steps):
            flush_buf.fill_(i & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            one_step(2000 + i)
            b.record(stream)
            torch.cuda.synchronize()
            t_total += a.elapsed_time(b) / 1e3
    else:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for i in range(steps):
            one_step(2000 + i)
        ev1.record(stream)
        torch.cuda.synchronize()
        t_total = ev0.elapsed_time(ev1) / 1e3
    # per-launch walk-kernel time: the library records CUDA events on the
    # stream around its walk launch (and after the sparse post-processing);
    # the same batches again, so the step counts are those of the timed ones
    graph.profile(True)
    kern_ms, post_ms = [], []
    total_steps = 0
    for i in range(steps):
        if flush_l2:
            flush_buf.fill_(i & 0xFF)
        one_step(2000 + i)
        wms, pms = graph.last_timings()
        kern_ms.append(wms)
        post_ms.append(pms)
        total_steps += int(steps_dev.item())
    graph.profile(False)
    if sampler:
        res["clocks"] = sampler.stop()
    steps_per_batch = total_steps / steps
    t_total, all_steps = replicas.reduce_timing(t_total, steps_per_batch * steps, world, dev)
    res.update(value=all_steps / t_total, ms_per_step=t_total / steps * 1e3, measured_steps_per_batch=steps_per_batch,
               gpu_launches=launches_per_step * steps)

    host = host_arrays(inp) if (rank == 0 and (not args.no_parity or not args.no_cpu)) else None
    # ---- parity: the last batch above (seed 2000 + steps - 1) against the oracle, untimed
    if not args.no_parity and outputs is not None and host is not None:
        t0 = time.perf_counter()
        ok, what = parity_sample(name, wl, host, replicas.replica_seed(2000 + steps - 1, rank), outputs,
                                 inp.get("per_query", 0))
        res["parity_checked"] = bool(ok)
        res["parity"] = "%s (%.1f s, untimed)" % (what, time.perf_counter() - t0)
    else:
        res["parity_checked"] = False

    # ---- e2e: through the C ABI with host buffers (pinned sources in, results out)
    h_src = src.cpu().pin_memory()
    h_steps = torch.zeros(1, dtype=torch.int64).pin_memory()
    if sparse:
        h_off = torch.empty(Q + 1, dtype=torch.int64).pin_memory()
        h_vert = torch.empty(cap, dtype=torch.int32).pin_memory()
        h_vcnt = torch.empty(cap, dtype=torch.int32).pin_memory()
    elif name != "ppr":
        h_paths = torch.empty((W, wl["length"]), dtype=torch.int32).pin_memory()  # the walks' result
    torch.cuda.synchronize()

    def e2e_step(i):
        if sparse:
            d = E.PPR(wl["tp"]).desc(replicas.replica_seed(3000 + i, rank))
            N.check(L.trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), _c(h_src), Q, per_q, _c(h_off),
                                           _c(h_vert), _c(h_vcnt), cap, _c(h_steps), 0, sp))
            return int(h_steps.item()), 8 * (Q + 1) + 8 * int(h_off[-1].item()) + 8
        elif name == "ppr":
            d = E.PPR(wl["tp"]).desc(replicas.replica_seed(3000 + i, rank))
            N.check(L.trw_ppr_batch(graph.handle, ctypes.byref(d), _c(h_src), Q, per_q, _c(counts), _c(h_steps),
                                    1, 0, sp))
            return int(h_steps.item()), 8
        d = app.desc(replicas.replica_seed(3000 + i, rank))
        N.check(L.trw_walk(graph.handle, ctypes.byref(d), _c(h_src), W, 0, _c(h_paths), wl["length"], None, None,
                           _c(h_steps), 0, sp))
        return int(h_steps.item()), h_paths.numel() * 4 + 8

    e2e_step(-1)  # untimed: the first host-buffer call allocates its staging and copy streams
    torch.cuda.synchronize()
    e2e_n = steps if headline else min(steps, 3)
    t0 = time.perf_counter()
    e2e_steps, d2h = 0, 0
    for i in range(e2e_n):
        s_i, b_i = e2e_step(i)
        e2e_steps += s_i
        d2h += b_i
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    res["e2e"] = {"value": e2e_steps / e2e_t, "unit": "steps/s", "h2d_bytes_per_step": int(h_src.numel() * 4),
                  "d2h_bytes_per_step": int(d2h / max(1, e2e_n))}

    # ---- plain forms (the comparison engine: one thread per walker, no refill)
    if not args.no_plain:
        reps = max(1, min(3, steps))
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for r in range(reps):
            one_step(4000 + r, engine="plain")
        b.record(stream)
        torch.cuda.synchronize()
        t1 = a.elapsed_time(b) / 1e3 / reps
        res["plain_one_launch"] = {"value": steps_per_batch / t1, "unit": "steps/s", "ms_per_step": t1 * 1e3,
                                   "form": "one launch over the whole batch, one thread per walker, no refill"}
        res["vs_plain_one_launch"] = res["value"] / res["plain_one_launch"]["value"]
        if name == "ppr":
            # one launch per query (the plain one-kernel-per-query form)
            a.record(stream)
            for r in range(reps):
                for qi in range(Q):
                    d = E.PPR(wl["tp"]).desc(4000 + r)
                    qsrc = ctypes.c_void_p(src.data_ptr() + 4 * qi)
                    if sparse:
                        N.check(L.trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), qsrc, 1, per_q, _c(offsets),
                                                       _c(vert), _c(vcnt), cap, _c(steps_dev), 1, sp))
                    else:
                        N.check(L.trw_ppr_batch(graph.handle, ctypes.byref(d), qsrc, 1, per_q,
                                                ctypes.c_void_p(counts.data_ptr() + 4 * qi * graph.n),
                                                _c(steps_dev), 1, 1, sp))
            b.record(stream)
            torch.cuda.synchronize()
            t2 = a.elapsed_time(b) / 1e3 / reps
            res["plain"] = {"value": steps_per_batch / t2, "unit": "steps/s", "ms_per_step": t2 * 1e3,
                            "form": "one launch per query, one thread per walker, no refill"}
        else:
            res["plain"] = res["plain_one_launch"]
        res["vs_plain"] = res["value"] / res["plain"]["value"]

    # ---- roofline of the walk kernel
    kmean = statistics.mean(kern_ms) / 1e3
    if name in BYTES_PER_STEP:
        bps = BYTES_PER_STEP[name]
    else:
        # Algorithmic bytes per move of the timed walks (the last batch's
        # paths, first 65536 walkers) under the kernel's own access pattern.
        sample = paths[:65536].cpu().numpy()
        if name == "node2vec":  # probes only where the kernel makes them (its draws, from the seed)
            bps = bytes_model.node2vec(sample, wl["length"], seed=replicas.replica_seed(2000 + steps - 1, rank),
                                       p=wl["p"], q=wl["q"], fat=graph.layout()[0] == 1)
        elif graph.indexes()[1] == 1:  # MetaPath answered from the label index
            bps = bytes_model.metapath_index(sample, inp["row"].cpu().numpy(), wl["length"],
                                             fat=graph.layout()[1] == 1)
        else:
            bps = bytes_model.metapath(sample, inp["row"].cpu().numpy(), wl["length"])
    achieved = steps_per_batch * bps / kmean / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    tkey = "ppr_dense" if name == "ppr" and not sparse else name
    traffic = TRAFFIC_BYTES_PER_STEP[tkey] * steps_per_batch if tkey in TRAFFIC_BYTES_PER_STEP else None
    res["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "traffic": traffic, "bytes_per_step": bps, "kernel_ms": kmean * 1e3,
                       "post_ms": statistics.mean(post_ms) if sparse else None,
                       "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}

    # ---- CPU baseline (rank 0 only)
    if host is not None and not args.no_cpu:
        cb = cpu_baseline(name, wl, host, inp.get("per_query", 0), args.cpu_seconds if headline else
                          args.cpu_seconds / 3)
        res["cpu_baseline"] = dict(cb, unit="steps/s", kind="port")
    graph.close()
    del inp, graph
    torch.cuda.empty_cache()
    return res


def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    res = measure(args.workload, args, args, dev, rank, world, args.steps, args.warmup, headline=True)
    side = {}
    if not args.no_workloads and args.workload == "ppr" and not args.scale and not args.queries:
        plain_args = SimpleNamespace(scale=None, queries=None)
        for name in SIDE_WORKLOADS:
            r = measure(name, args, plain_args, dev, rank, world, args.side_steps, max(3, args.warmup // 2),
                        headline=False)
            side[name] = {k: r[k] for k in ("config", "value", "ms_per_step", "e2e", "roofline", "plain",
                                             "vs_plain", "parity_checked", "parity", "cpu_baseline", "engine")
                          if k in r}
    if rank == 0:
        line = {
            "metric": "walk_steps_per_s", "value": res["value"], "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
            "data": "synthetic (seeded generator, no dataset)",
            "config": res["config"],
            "engine": res["engine"],
            "measured_steps_per_batch": res["measured_steps_per_batch"],
            "kernel_timing": "walk-kernel CUDA events recorded by the library on the launch stream",
            "gpu_launches": res["gpu_launches"], "clocks": res.get("clocks"), "e2e": res["e2e"],
            "roofline": res["roofline"], "plain": res.get("plain"), "vs_plain": res.get("vs_plain"),
            "plain_one_launch": res.get("plain_one_launch"), "vs_plain_one_launch": res.get("vs_plain_one_launch"),
            "parity_checked": res["parity_checked"], "parity": res.get("parity"),
            "cpu_baseline": res.get("cpu_baseline"),
        }
        if side:
            line["workloads"] = side
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_serving(args):
    """Serving mix: Poisson arrivals at swept rates on a resident R-MAT graph
    (alias + ITS tables, edge set and label index built), apps uniform over
    PPR / DeepWalk / Node2Vec / MetaPath, walkers log-uniform in [1e3, 1e6],
    lengths uniform in [5, 80].  Per rate: offered and achieved request rates,
    steps/s, p50 / p99 latency (submit -> results complete in HBM) and the
    number of batches (persistent launches per kernel) the loop formed.
    Sources come from one pool of random non-isolated vertices drawn once,
    so submitting a request costs no sampling on the host."""
    import torch
    from thunderrw_gb300 import engine as E
    from thunderrw_gb300 import generators as G
    from thunderrw_gb300.serving import Server

    torch.cuda.set_device(0)
    scale = args.scale or 25
    g = G.make_graph("rmat", 1 << scale, 32, seed=20240601, device="cuda", labels=5)
    graph = E.Graph(g["row"], g["adj"], g["weight"], g["label"])
    pool = G.random_sources(g["row"], 1 << 22, seed=17).cpu().numpy()
    del g
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    graph.build_tables("alias", "edge")
    graph.build_tables("its", "edge")
    indexes = graph.build_indexes()  # Node2Vec edge set, MetaPath label index: no request builds them
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    apps = [None, E.DeepWalk, lambda L: E.Node2Vec(L, 2.0, 0.5), lambda L: E.MetaPath(L, [0, 1, 2, 3, 4])]
    results = []
    for rate in [float(x) for x in args.rates.split(",")]:
        n = int(rate * args.serve_seconds) + 1
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
        kinds = rng.integers(0, 4, size=n)
        walkers = np.exp(rng.uniform(np.log(1e3), np.log(1e6), size=n)).astype(np.int64)
        lengths = rng.integers(5, 81, size=n)
        starts = rng.integers(0, pool.size - 1_000_000, size=n)
        seeds = rng.integers(1, 1 << 62, size=n)
        srv = Server(graph, max_inflight=args.inflight)
        tickets = []
        done = threading.Event()

        def collector():
            i = 0
            while not (done.is_set() and i >= len(tickets)):
                if i < len(tickets):
                    srv.wait(tickets[i])
                    srv.release(tickets[i])
                    i += 1
                else:
                    time.sleep(0.0002)

        th = threading.Thread(target=collector)
        th.start()
        t_start = time.perf_counter()
        for i in range(n):
            while time.perf_counter() - t_start < arrivals[i]:
                pass
            k = int(kinds[i])
            if k == 0:
                tickets.append(srv.submit_ppr(pool[starts[i]:starts[i] + 1], int(walkers[i]), tp=0.2, seed=int(seeds[i])))
            else:
                tickets.append(srv.submit_walk(apps[k](int(lengths[i])), pool[starts[i]:starts[i] + int(walkers[i])],
                                               seed=int(seeds[i])))
        offered_s = time.perf_counter() - t_start
        done.set()
        th.join()
        st = srv.stats()
        srv.stop()
        results.append({"rate_req_s": rate, "requests": n, "offered_req_s": n / offered_s,
                        "achieved_req_s": st["completed"] / st["elapsed_s"], "completed": st["completed"],
                        "failed": st["failed"], "batches": st["batches"], "p50_ms": st["p50_ms"],
                        "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
                        "steps_per_s": st["steps"] / st["elapsed_s"], "elapsed_s": st["elapsed_s"]})
        print(json.dumps(results[-1]), file=sys.stderr, flush=True)
    best = max(results, key=lambda r: r["steps_per_s"])
    line = {"metric": "walk_steps_per_s", "value": best["steps_per_s"], "unit": "steps/s", "n_gpus": 1,
            "steps": len(results), "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32+f64", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "serving mix rmat N=2^%d deg=32, 5 labels, alias+ITS tables, edge set and label "
                                   "index resident; PPR/DeepWalk/Node2Vec/MetaPath uniform, walkers log-uniform "
                                   "1e3-1e6, L 5-80, Poisson arrivals" % scale,
                       "n": graph.n, "e": graph.e, "table_build_s": build_s, "max_inflight": args.inflight,
                       "indexes": {"edge_set": indexes[0], "label_index": indexes[1],
                                   "fat_adjacency": graph.layout()[0]}},
            "serving": results}
    print(json.dumps(line), flush=True)
    graph.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
