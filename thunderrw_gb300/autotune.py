"""Launch-shape autotuner.

The reference fixes its ring (RING_SIZE = 64 slots per thread, 32 search
frames, creeper.h / types.h) at compile time.  Here the equivalent knobs are
runtime launch shapes of the persistent engine: walkers in flight per lane
(the ring depth R, 1/2/4/8) and CTAs per SM, or the plain form (one thread
per walker, no refill; shape (-1, 0)), which some fixed-length walks run
fastest in.  Which shape is fastest depends
on the graph's degree profile and the app: sparse-table PPR and max-weight
rejection want R = 1, static alias R = 4 on large batches, and a batch of
about one walker per lane (DeepWalk on Chung-Lu 2^18) runs fastest with 4
CTAs per SM instead of the 6 that fit.  `tune` times each candidate shape on a sample of the
caller's own workload with CUDA events and sets the fastest on the graph
(`trw_set_engine_shape`), so later calls with the same sampler use it.
Walks are a function of (seed, walker, step) only, so the shape never changes
results, only their speed.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import engine as E

WARP_FAMILY = {"its", "alias", "rejection"}  # dynamic mode: one warp per walker step, no ring


@dataclass
class TuneResult:
    sampler: str                     # the engine-shape slot that was tuned
    best: Tuple[int, int]            # (walkers per lane, CTAs per SM); 0 = automatic
    best_ms: float
    timings: Dict[Tuple[int, int], float] = field(default_factory=dict)
    walkers: int = 0                 # walkers in the timed sample


def _slot(app: E.App, mode: Optional[str], sampler: Optional[str]) -> Tuple[str, bool]:
    m = mode or app.mode
    s = sampler or app.sampler
    if m == "uniform":
        return "uniform", False
    if app.name == "metapath" and m == "dynamic" and s == "its":
        return s, False  # the label index runs on the ring engine (the row scan ignores the ring)
    if app.name in ("deepwalk", "genericwalk", "ppr"):
        return s, False  # walker-independent weights: dynamic mode runs on the static tables
    return s, (m == "dynamic" and s in WARP_FAMILY)


def tune(graph: E.Graph, app: E.App, sources, walkers_per_query: int = 0, mode: Optional[str] = None,
         sampler: Optional[str] = None, rings: Sequence[int] = (1, 2, 4, 8),
         ctas: Sequence[int] = (0, 2, 4, 8), sample_walkers: Optional[int] = None, repeats: int = 3,
         record_paths: bool = True, seed: int = 12345, apply: bool = True,
         tolerance: float = 0.03, plain: bool = True) -> TuneResult:
    """Times every (ring, CTAs/SM) candidate on a sample of the workload and
    keeps the fastest.  `walkers_per_query` > 0 tunes sparse batched PPR
    (`sources` are then the queries).  The sample keeps at least 16 walkers
    per lane of the GPU (the engine's steady state), or the whole workload
    if it is smaller.  The automatic shape (0, 0) is timed too and kept
    unless a candidate beats it by more than `tolerance`, so timing noise
    does not move the shape."""
    dev = graph.device
    src = torch.as_tensor(sources).to(device=dev, dtype=torch.int32).flatten()
    slot, warp_family = _slot(app, mode, sampler)
    props = torch.cuda.get_device_properties(dev)
    lanes = props.multi_processor_count * 2048
    target = sample_walkers or 16 * lanes
    if walkers_per_query > 0:
        q = max(1, min(src.numel(), -(-target // walkers_per_query)))
        src = src[:q]
        walkers = q * walkers_per_query
    else:
        src = src[:min(src.numel(), target)]
        walkers = src.numel()
    cands: List[Tuple[int, int]] = [(0, 0)]
    for r in ((0,) if warp_family else rings):
        for c in ctas:
            if (r, c) not in cands:
                cands.append((r, c))
    if plain and not warp_family:
        cands.append((-1, 0))
    old = graph.engine_shape(slot)
    stream = torch.cuda.current_stream(dev)

    def run(i):
        if walkers_per_query > 0:
            E.ppr_batch_sparse(graph, src, walkers_per_query, tp=app.tp, seed=seed + i, stream=stream)
        else:
            E.compute(graph, src, app, mode=mode, sampler=sampler, seed=seed + i, record_paths=record_paths,
                      stream=stream)

    timings: Dict[Tuple[int, int], float] = {}
    try:
        for r, c in cands:
            graph.set_engine_shape(slot, r, c)
            run(0)  # warm-up (and lazy table builds / allocations)
            torch.cuda.synchronize(dev)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for i in range(repeats):
                run(1 + i)
            b.record(stream)
            torch.cuda.synchronize(dev)
            timings[(r, c)] = a.elapsed_time(b) / repeats
    finally:
        graph.set_engine_shape(slot, *old)
    best = min(timings, key=timings.get)
    if timings[(0, 0)] <= timings[best] * (1.0 + tolerance):
        best = (0, 0)
    if apply:
        graph.set_engine_shape(slot, *best)
    return TuneResult(slot, best, timings[best], timings, walkers)
