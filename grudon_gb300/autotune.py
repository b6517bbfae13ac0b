"""Schedule autotuner for the device-driven round loop.

Candidates vary only schedule knobs — the number of memory partitions of the
layout, the dense/sparse dirty-tracking threshold and the push grid size —
none of which changes any result.  Each candidate is timed on the real
workload (warm-up run, then timed runs with CUDA events on the ctx stream)
and the fastest is kept.
"""
from __future__ import annotations

import itertools
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence

from . import Context, Graph


@dataclass
class Candidate:
    num_memory: int = 1
    dense_div: int = 32
    push_blocks_per_sm: int = 0

    def params(self) -> dict:
        return {"dense_div": self.dense_div, "push_blocks_per_sm": self.push_blocks_per_sm}


@dataclass
class TuneResult:
    best: Candidate
    best_ms: float
    table: List[dict] = field(default_factory=list)


def default_space(max_memory: int = 3) -> List[Candidate]:
    mems = [m for m in (1, 3) if m <= max_memory]
    return [Candidate(m, d, b) for m, d, b in itertools.product(mems, (8, 32, 128), (0, 2, 8))]


def _time_runs(ctx: Context, prepare: Callable[[Context], None], reps: int) -> float:
    import torch
    s = torch.cuda.ExternalStream(ctx.stream())
    best = float("inf")
    for _ in range(reps):
        prepare(ctx)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        ctx.run()
        e1.record(s)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune(graph: Graph, algo: int, prepare: Callable[[Context], None], space: Optional[Sequence[Candidate]] = None,
         set_algo_kwargs: Optional[Dict] = None, device: int = 0, reps: int = 3,
         partitioner: Optional[Callable[[Graph, int], object]] = None) -> TuneResult:
    """prepare(ctx) must leave the ctx ready to run (it calls init / init_sources)."""
    space = list(space or default_space())
    kw = dict(set_algo_kwargs or {})
    table = []
    by_m: Dict[int, Context] = {}
    try:
        for cand in space:
            if cand.num_memory not in by_m:
                part = None
                if cand.num_memory > 1:
                    part = (partitioner or (lambda G, m: G.partition_edge_balanced(m)))(graph, cand.num_memory)
                by_m[cand.num_memory] = Context(graph, part, cand.num_memory, device)
            ctx = by_m[cand.num_memory]
            ctx.set_algo(algo, **kw, **cand.params())
            prepare(ctx)
            ctx.run()  # warm-up (also builds the loop graph)
            ms = _time_runs(ctx, prepare, reps)
            table.append({**cand.__dict__, "ms": ms})
    finally:
        for c in by_m.values():
            c.close()
    best = min(table, key=lambda r: r["ms"])
    return TuneResult(Candidate(best["num_memory"], best["dense_div"], best["push_blocks_per_sm"]), best["ms"], table)
