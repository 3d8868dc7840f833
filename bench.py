#!/usr/bin/env python
"""Walk-steps/s benchmark of the GB300 random-walk engine.

Default workload (the batched-PPR configuration): R-MAT graph (a,b,c =
0.57,0.19,0.19), N = 2^22 vertices, average degree 32 before symmetrisation,
undirected int32 CSR; 4096 queries x 10^4 walkers whose sources are drawn
uniformly among non-isolated vertices; uniform sampling, termination
probability 0.2 after every move (geometric lengths, mean 5); output: int32
visit counts per query (4096 x N, zeroed inside every step).  One step = one
whole batch through trw_ppr_batch.  Inputs (adjacency 0.5 GB, counts 64 GiB)
are far larger than the 129 MB L2, so no separate flush is needed.

Prints one JSON line (rank 0).  --impl reference times the reference's CPU
algorithm (the step-interleaved C++ oracle port of creeper.h's ring) on the
host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ppr", choices=sorted(WORKLOADS) + ["serving"])
    ap.add_argument("--rates", default="50,200,800", help="serving: arrival rates (requests/s)")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--queries", type=int, default=None, help="override the query count (small runs)")
    ap.add_argument("--scale", type=int, default=None, help="override log2(N) (small runs)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-tune", action="store_true", help="keep the automatic launch shape (no autotuning)")
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
# workload construction
# ---------------------------------------------------------------------------

def workload_name(wl, args):
    """The workload's name, with any size override spelled out."""
    over = []
    if args.scale:
        over.append("N=2^%d" % args.scale)
    if args.queries:
        over.append("%d queries" % args.queries)
    return wl["name"] + (" [reduced: %s]" % ", ".join(over) if over else "")


def build_inputs(wl, args, device, rank=0):
    """The workload's graph (the same on every rank) and rank's own sources."""
    import torch
    from thunderrw_gb300 import generators as G
    n = 1 << args.scale if args.scale else wl["n"]
    g = G.make_graph(wl["kind"], n, wl["deg"], seed=20240601, device=device,
                     weights=wl["kind"] != "rmat" or "length" in wl, labels=wl.get("labels", 0))
    out = {"n": n, "row": g["row"], "adj": g["adj"], "weight": g["weight"], "label": g["label"]}
    if "queries" in wl:
        q = args.queries or wl["queries"]
        out["sources"] = G.random_sources(g["row"], q, seed=replicas.replica_seed(7, rank) & 0x7FFFFFFF)
        out["per_query"] = wl["per_query"]
    elif "walkers" in wl:
        out["sources"] = G.random_sources(g["row"], wl["walkers"], seed=replicas.replica_seed(7, rank) & 0x7FFFFFFF)
    else:
        out["sources"] = G.all_sources(g["row"], seed=0)
    if torch.device(device).type == "cuda":
        torch.cuda.synchronize()
    return out


def cpu_baseline(wl_name, wl, row, adj, weight, sources, per_query, seconds, threads, label=None):
    """The step-interleaved CPU port (oracle) on a bounded sample of the same
    workload, on all host threads.  Returns (steps/s, sample description)."""
    from oracle import oracle as O
    og = O.Graph(row, adj, weight, label)
    ncores = threads or os.cpu_count()
    if wl_name == "ppr":
        d = O.make_desc("ppr", "uniform", "uniform", length=1, tp=wl["tp"], seed=11)
        chunk = 64  # queries per pass; each pass zeroes and fills a chunk x N count block
        counts = np.zeros((chunk, og.n), dtype=np.int32)
        counts.fill(1)  # touch every page once, outside the timed passes
        total_steps, total_t, done_q = 0, 0.0, 0
        src = np.asarray(sources, dtype=np.int32)
        while total_t < seconds:  # the batch again (fresh walker ids) until the budget is spent
            at = done_q % src.size
            qs = src[at:at + chunk]
            t0 = time.perf_counter()
            counts[: qs.size].fill(0)
            r = O.walk(og, d, qs, per_query=per_query, id_base=done_q * per_query, want_lengths=False,
                       num_queries=qs.size, threads=ncores, interleaved=True, ring=64, out_counts=counts)
            total_t += time.perf_counter() - t0
            total_steps += r["steps"]
            done_q += qs.size
        sample = ("step-interleaved C++ port of the reference ring (64 walkers per thread), "
                  "%d queries x %d walkers (%d steps, %.2f passes over the batch) in %.1f s" % (
                      done_q, per_query, total_steps, done_q / src.size, total_t))
        return total_steps / total_t, sample, ncores
    if wl_name == "deepwalk":
        og.build_tables("alias", 0)
        d = O.make_desc("deepwalk", "static", "alias", length=wl["length"], seed=11)
    else:  # dynamic samplers, on the same step-interleaved ring
        d = O.make_desc(wl_name, "dynamic", "maxweight_rejection" if wl_name == "node2vec" else "its",
                        length=wl["length"], p=wl.get("p", 1.0), q=wl.get("q", 1.0), schema=wl.get("schema"), seed=11)
    src = np.asarray(sources, dtype=np.int32)
    total_steps, total_t, done = 0, 0.0, 0
    chunk = 1 << 16
    paths = None
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
        paths = r["paths"]
    del paths
    form = "step-interleaved C++ port of the reference ring (64 walkers per thread)"
    return total_steps / total_t, "%s, %d walkers x %d steps (%d steps, %.2f passes over the workload) in %.1f s" % (
        form, done, wl["length"] - 1, total_steps, done / src.size, total_t), ncores


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
    row = inp["row"].cpu().numpy()
    adj = inp["adj"].cpu().numpy()
    weight = inp["weight"].cpu().numpy() if inp["weight"] is not None else None
    label = inp["label"].cpu().numpy() if inp.get("label") is not None else None
    src = inp["sources"].cpu().numpy()
    per_q = inp.get("per_query", 0)
    del inp
    if have_gpu:
        torch.cuda.empty_cache()
    vals = []
    sample = ""
    cores = os.cpu_count()
    for i in range(args.warmup + args.steps):
        v, sample, cores = cpu_baseline(args.workload, wl, row, adj, weight, src, per_q,
                                        max(2.0, 20.0 / max(1, args.warmup + args.steps)), 0, label=label)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": "walk_steps_per_s", "value": value, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic",
        "config": {"workload": workload_name(wl, args)},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port",
                         "sample": "per step: " + sample},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from thunderrw_gb300 import _native as N
    from thunderrw_gb300 import engine as E

    wl = WORKLOADS[args.workload]
    inp = build_inputs(wl, args, dev, rank)
    graph = E.Graph(inp["row"], inp["adj"], inp["weight"], inp.get("label"))
    stream = torch.cuda.current_stream(dev)
    L = N.load()
    import ctypes

    sparse = args.workload == "ppr" and not args.dense
    out_bytes = 0
    if args.workload == "ppr":
        Q = inp["sources"].numel()
        per_q = inp["per_query"]
        steps_dev = torch.zeros(1, dtype=torch.int64, device=dev)
        src = inp["sources"]
        if sparse:
            # size the CSR output from one untimed batch (same shape, other seed)
            probe = E.ppr_batch_sparse(graph, src, per_q, tp=wl["tp"], seed=999)
            cap = int(int(probe.offsets[-1].item()) * 1.25) + 1024
            del probe
            offsets = torch.empty(Q + 1, dtype=torch.int64, device=dev)
            vert = torch.empty(cap, dtype=torch.int32, device=dev)
            vcnt = torch.empty(cap, dtype=torch.int32, device=dev)
            counts = None

            def one_step(seed, engine="persistent"):
                d = E.PPR(wl["tp"]).desc(replicas.replica_seed(seed, rank))
                N.check(L.trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), ctypes.c_void_p(src.data_ptr()), Q,
                                               per_q, ctypes.c_void_p(offsets.data_ptr()),
                                               ctypes.c_void_p(vert.data_ptr()), ctypes.c_void_p(vcnt.data_ptr()), cap,
                                               ctypes.c_void_p(steps_dev.data_ptr()), N.ENGINES[engine],
                                               ctypes.c_void_p(stream.cuda_stream)))
        else:
            counts = torch.empty((Q, graph.n), dtype=torch.int32, device=dev)

            def one_step(seed, engine="persistent"):
                d = E.PPR(wl["tp"]).desc(replicas.replica_seed(seed, rank))
                N.check(L.trw_ppr_batch(graph.handle, ctypes.byref(d), ctypes.c_void_p(src.data_ptr()), Q, per_q,
                                        ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(steps_dev.data_ptr()),
                                        1, N.ENGINES[engine], ctypes.c_void_p(stream.cuda_stream)))
    else:
        src = inp["sources"]
        W = src.numel()
        Lw = wl["length"]
        paths = torch.empty((W, Lw), dtype=torch.int32, device=dev)
        lengths = torch.empty(W, dtype=torch.int32, device=dev)
        steps_dev = torch.zeros(1, dtype=torch.int64, device=dev)
        counts = None
        app = {"deepwalk": E.DeepWalk(Lw),
               "node2vec": E.Node2Vec(Lw, wl.get("p", 2.0), wl.get("q", 0.5)),
               "metapath": E.MetaPath(Lw, wl.get("schema", [0, 1, 2, 3, 4]))}[args.workload]
        if args.workload == "deepwalk":
            graph.build_tables("alias", "edge")

        def one_step(seed, engine="persistent"):
            d = app.desc(replicas.replica_seed(seed, rank))
            N.check(L.trw_walk(graph.handle, ctypes.byref(d), ctypes.c_void_p(src.data_ptr()), W, 0,
                               ctypes.c_void_p(paths.data_ptr()), Lw, ctypes.c_void_p(lengths.data_ptr()), None,
                               ctypes.c_void_p(steps_dev.data_ptr()), N.ENGINES[engine],
                               ctypes.c_void_p(stream.cuda_stream)))

    # ---- launch shape: tuned once on a sample of this workload, as a user
    # would (thunderrw_gb300/autotune.py), outside every timed region
    shape = None
    if args.shape:
        slot = "uniform" if args.workload == "ppr" else app.sampler
        r, c = (int(x) for x in args.shape.split(","))
        graph.set_engine_shape(slot, r, c)
        shape = {"slot": slot, "walkers_per_lane": r, "ctas_per_sm": c, "set_by": "--shape"}
    elif not args.no_tune:
        from thunderrw_gb300 import autotune
        if args.workload == "ppr":
            res = autotune.tune(graph, E.PPR(wl["tp"]), src, walkers_per_query=per_q, rings=(1, 2), ctas=(0, 4),
                                repeats=2)
        else:
            res = autotune.tune(graph, app, src, rings=(1, 2, 4), ctas=(0, 2, 4), repeats=2)
        shape = {"slot": res.sampler, "walkers_per_lane": res.best[0], "ctas_per_sm": res.best[1],
                 "tuned_on_walkers": res.walkers, "candidates": len(res.timings)}
        torch.cuda.synchronize()

    # ---- warm-up
    for i in range(args.warmup):
        one_step(1000 + i)
    torch.cuda.synchronize()

    # ---- timed region: K whole batches, fresh seeds
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    total_steps = 0
    # Working sets that fit in L2 (the 129 MB L2) are flushed between timed
    # steps by writing a 512 MB buffer outside the events; larger inputs need
    # no flush.
    working = graph.e * 4 + graph.n * 8 + (graph.e * 16 if args.workload == "deepwalk" else 0)
    flush_l2 = working < 2 * 129e6
    flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device=dev) if flush_l2 else None
    if flush_l2:
        t_total = 0.0
        for i in range(args.steps):
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
        for i in range(args.steps):
            one_step(2000 + i)
        ev1.record(stream)
        torch.cuda.synchronize()
        t_total = ev0.elapsed_time(ev1) / 1e3
    # per-launch walk-kernel time: the library records CUDA events on the
    # stream around its walk launch (and after the sparse post-processing)
    graph.profile(True)
    kern_ms, post_ms = [], []
    for i in range(args.steps):
        if flush_l2:
            flush_buf.fill_(i & 0xFF)
        one_step(2000 + i)
        wms, pms = graph.last_timings()
        kern_ms.append(wms)
        post_ms.append(pms)
        total_steps += int(steps_dev.item())
    graph.profile(False)
    clocks = sampler.stop()
    steps_per_batch = total_steps / args.steps
    t_total, all_steps = replicas.reduce_timing(t_total, steps_per_batch * args.steps, world, dev)
    value = all_steps / t_total

    # ---- e2e: through the C ABI with host buffers (pinned sources in, results out)
    h_src = src.cpu().pin_memory()
    h_steps = torch.zeros(1, dtype=torch.int64).pin_memory()
    if sparse:
        h_off = torch.empty(Q + 1, dtype=torch.int64).pin_memory()
        h_vert = torch.empty(cap, dtype=torch.int32).pin_memory()
        h_vcnt = torch.empty(cap, dtype=torch.int32).pin_memory()
    elif args.workload != "ppr":
        h_paths = torch.empty((W, wl["length"]), dtype=torch.int32).pin_memory()  # the walks' result
    torch.cuda.synchronize()

    def e2e_step(i):
        if args.workload == "ppr" and sparse:
            d = E.PPR(wl["tp"]).desc(replicas.replica_seed(3000 + i, rank))
            N.check(L.trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), ctypes.c_void_p(h_src.data_ptr()), Q, per_q,
                                           ctypes.c_void_p(h_off.data_ptr()), ctypes.c_void_p(h_vert.data_ptr()),
                                           ctypes.c_void_p(h_vcnt.data_ptr()), cap, ctypes.c_void_p(h_steps.data_ptr()),
                                           0, ctypes.c_void_p(stream.cuda_stream)))
            return int(h_steps.item()), 8 * (Q + 1) + 8 * int(h_off[-1].item()) + 8
        elif args.workload == "ppr":
            d = E.PPR(wl["tp"]).desc(replicas.replica_seed(3000 + i, rank))
            N.check(L.trw_ppr_batch(graph.handle, ctypes.byref(d), ctypes.c_void_p(h_src.data_ptr()), Q, per_q,
                                    ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(h_steps.data_ptr()), 1, 0,
                                    ctypes.c_void_p(stream.cuda_stream)))
            return int(h_steps.item()), 8
        d = app.desc(replicas.replica_seed(3000 + i, rank))
        N.check(L.trw_walk(graph.handle, ctypes.byref(d), ctypes.c_void_p(h_src.data_ptr()), W, 0,
                           ctypes.c_void_p(h_paths.data_ptr()), wl["length"], None, None,
                           ctypes.c_void_p(h_steps.data_ptr()), 0, ctypes.c_void_p(stream.cuda_stream)))
        return int(h_steps.item()), h_paths.numel() * 4 + 8

    e2e_step(-1)  # untimed: the first host-buffer call allocates its staging and copy streams
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps, d2h = 0, 0
    for i in range(args.steps):
        s_i, b_i = e2e_step(i)
        e2e_steps += s_i
        d2h += b_i
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    e2e = {"value": e2e_steps / e2e_t, "unit": "steps/s", "h2d_bytes_per_step": int(h_src.numel() * 4),
           "d2h_bytes_per_step": int(d2h / max(1, args.steps))}

    # ---- plain one-launch-per-query form (the comparison engine)
    plain = None
    if not args.no_plain:
        reps = max(1, min(3, args.steps))
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if args.workload == "ppr":
            # one launch per query, one thread per walker, no refill
            a.record(stream)
            for r in range(reps):
                for qi in range(Q):
                    d = E.PPR(wl["tp"]).desc(4000 + r)
                    qsrc = ctypes.c_void_p(src.data_ptr() + 4 * qi)
                    if sparse:
                        N.check(L.trw_ppr_batch_sparse(graph.handle, ctypes.byref(d), qsrc, 1, per_q,
                                                       ctypes.c_void_p(offsets.data_ptr()),
                                                       ctypes.c_void_p(vert.data_ptr()),
                                                       ctypes.c_void_p(vcnt.data_ptr()), cap,
                                                       ctypes.c_void_p(steps_dev.data_ptr()), 1,
                                                       ctypes.c_void_p(stream.cuda_stream)))
                    else:
                        N.check(L.trw_ppr_batch(graph.handle, ctypes.byref(d), qsrc, 1, per_q,
                                                ctypes.c_void_p(counts.data_ptr() + 4 * qi * graph.n),
                                                ctypes.c_void_p(steps_dev.data_ptr()), 1, 1,
                                                ctypes.c_void_p(stream.cuda_stream)))
            b.record(stream)
            torch.cuda.synchronize()
        else:
            a.record(stream)
            for r in range(reps):
                one_step(4000 + r, engine="plain")
            b.record(stream)
            torch.cuda.synchronize()
        plain_t = a.elapsed_time(b) / 1e3 / reps
        plain = {"value": steps_per_batch / plain_t, "unit": "steps/s", "ms_per_step": plain_t * 1e3,
                 "form": "one thread per walker, one launch per query, no refill"}

    # ---- roofline of the walk kernel
    kmean = statistics.mean(kern_ms) / 1e3
    if args.workload in BYTES_PER_STEP:
        bps = BYTES_PER_STEP[args.workload]
    else:
        # Algorithmic bytes per move of the timed walks (the last batch's
        # paths, first 65536 walkers) under the kernel's own access pattern.
        sample = paths[:65536].cpu().numpy()
        if args.workload == "node2vec":
            bps = bytes_model.node2vec(sample, wl["length"])
        elif graph.indexes()[1] == 1:  # MetaPath answered from the label index
            bps = bytes_model.metapath_index(sample, inp["row"].cpu().numpy(), wl["length"])
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
    traffic = None
    # DRAM bytes per step from the committed ncu summary of the same kernel,
    # scaled to this launch by its step count
    import glob
    import re
    for md in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        key = "ppr_dense" if args.workload == "ppr" and not sparse else args.workload
        m = re.search(r"traffic_bytes_per_step_%s = ([0-9.]+)" % key, open(md).read())
        if m:
            traffic = float(m.group(1)) * steps_per_batch
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "bytes_per_step": bps, "kernel_ms": kmean * 1e3,
            "post_ms": statistics.mean(post_ms) if sparse else None,
            "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        row = inp["row"].cpu().numpy()
        adj = inp["adj"].cpu().numpy()
        wt = inp["weight"].cpu().numpy() if inp["weight"] is not None else None
        lab = inp["label"].cpu().numpy() if inp.get("label") is not None else None
        v, sample, cores = cpu_baseline(args.workload, wl, row, adj, wt, src.cpu().numpy(),
                                        inp.get("per_query", 0), args.cpu_seconds, 0, label=lab)
        cpu = {"value": v, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample}

    if rank == 0:
        line = {
            "metric": "walk_steps_per_s", "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": workload_name(wl, args), "n": graph.n, "e": graph.e,
                       "steps_per_batch": steps_per_batch, "engine": "persistent",
                       "launch_shape": shape or "automatic (0 = automatic)",
                       "counts": ("dense int32 [Q][N], zeroed every step" if args.workload == "ppr" and not sparse
                                  else "sparse CSR per query (offsets, vertex, int32 count)")
                       if args.workload == "ppr" else None,
                       "l2": ("L2 flushed between timed steps (512 MB write outside the events)" if flush_l2 else
                              "inputs larger than L2 (adjacency %.2f GB, counts %.1f GB), no flush" % (
                                  graph.e * 4 / 1e9, (counts.numel() * 4 / 1e9) if counts is not None else 0))},
            "kernel_timing": "walk-kernel CUDA events recorded by the library on the launch stream",
            "gpu_launches": args.steps, "clocks": clocks, "e2e": e2e, "roofline": roof,
            "plain": plain, "vs_plain": (value / plain["value"]) if plain else None, "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    graph.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_serving(args):
    """Serving mix: Poisson arrivals at swept rates on a resident R-MAT graph
    (alias + ITS tables, edge set and label index built), apps uniform over PPR / DeepWalk / Node2Vec /
    MetaPath, walkers log-uniform in [1e3, 1e6], lengths uniform in [5, 80].
    Reports p50 / p99 latency (submit -> results complete in HBM) and steps/s
    per arrival rate."""
    import threading
    import torch
    from thunderrw_gb300 import engine as E
    from thunderrw_gb300 import generators as G
    from thunderrw_gb300.serving import Server

    torch.cuda.set_device(0)
    scale = args.scale or 25
    g = G.make_graph("rmat", 1 << scale, 32, seed=20240601, device="cuda", labels=5)
    graph = E.Graph(g["row"], g["adj"], g["weight"], g["label"])
    nz = torch.nonzero(g["row"][1:] - g["row"][:-1]).flatten().to(torch.int32).cpu().numpy()
    del g
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    graph.build_tables("alias", "edge")
    graph.build_tables("its", "edge")
    indexes = graph.build_indexes()  # Node2Vec edge set, MetaPath label index: no request builds them
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    results = []
    for rate in [float(x) for x in args.rates.split(",")]:
        srv = Server(graph, max_inflight=8)
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
                    time.sleep(0.0005)

        th = threading.Thread(target=collector)
        th.start()
        t_start = time.perf_counter()
        nreq = 0
        while time.perf_counter() - t_start < args.serve_seconds:
            kind = rng.integers(0, 4)
            walkers = int(np.exp(rng.uniform(np.log(1e3), np.log(1e6))))
            length = int(rng.integers(5, 81))
            seed = int(rng.integers(1, 1 << 62))
            if kind == 0:
                tickets.append(srv.submit_ppr(rng.choice(nz, size=1), walkers, tp=0.2, seed=seed))
            else:
                app = [None, E.DeepWalk(length), E.Node2Vec(length, 2.0, 0.5), E.MetaPath(length, [0, 1, 2, 3, 4])][kind]
                tickets.append(srv.submit_walk(app, rng.choice(nz, size=walkers), seed=seed))
            nreq += 1
            time.sleep(rng.exponential(1.0 / rate))
        done.set()
        th.join()
        st = srv.stats()
        srv.stop()
        results.append({"rate_req_s": rate, "requests": nreq, "completed": st["completed"], "failed": st["failed"],
                        "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
                        "steps_per_s": st["steps"] / st["elapsed_s"], "elapsed_s": st["elapsed_s"]})
        print(json.dumps(results[-1]), file=sys.stderr, flush=True)
    best = max(results, key=lambda r: r["steps_per_s"])
    line = {"metric": "walk_steps_per_s", "value": best["steps_per_s"], "unit": "steps/s", "n_gpus": 1,
            "steps": len(results), "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32+f64", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "serving mix rmat N=2^%d deg=32, 5 labels, alias+ITS tables, edge set and label index resident" % scale,
                       "n": graph.n, "e": graph.e, "table_build_s": build_s,
                       "indexes": {"edge_set": indexes[0], "label_index": indexes[1]}},
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
