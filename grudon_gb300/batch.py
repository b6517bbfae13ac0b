"""Batched workloads on one GPU: many graphs, or many SSSP sources, in one run.

The graphs of a batch are laid out as one disjoint union (vertex ids of graph
i shifted by base_i), so every round's kernels cover the whole batch and the
whole batch runs as one device-driven CUDA-graph launch per algorithm.  No
edge crosses two graphs, so per-graph results are exact restrictions of the
union's:
  * CC labels of graph i are the union labels minus base_i (the minimum gid of
    a component never leaves the component);
  * SSSP from source s in copy i is the union's distance with every copy's
    source seeded (grd_init_sources);
  * PageRank is computed per vertex from in-neighbours only.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from . import Context, Graph, GRD_CC, GRD_PR_PULL, GRD_SSSP_W, rmat_seed

ER_D = 0.05


@dataclass(frozen=True)
class GraphSpec:
    kind: str  # "rmat" or "er"
    scale: int
    edge_factor: int
    a: float
    seed: int

    @property
    def abc(self):
        b = (1.0 - self.a - ER_D) / 2.0
        return self.a, b, b


def batch_spec(n: int = 512, seed: int = 0x62617463, lo: int = 10, hi: int = 18) -> List[GraphSpec]:
    """Scales log-uniform in [lo, hi] (rounded), edge factor uniform in
    {4, 8, 16, 32}; even indices RMAT with a ~ U[0.45, 0.65], b = c =
    (1 - a - 0.05)/2, d = 0.05; odd indices Erdos-Renyi."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        scale = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        ef = int(rng.choice([4, 8, 16, 32]))
        a = float(rng.uniform(0.45, 0.65))
        out.append(GraphSpec("rmat" if i % 2 == 0 else "er", scale, ef, a, int(rng.integers(1, 2**62))))
    return out


def make_graph(spec: GraphSpec, symmetrize: bool = False, weighted: bool = False, threads: int = 0) -> Graph:
    if spec.kind == "rmat":
        a, b, c = spec.abc
        return Graph.rmat(spec.scale, spec.edge_factor, a, b, c, seed=spec.seed, symmetrize=symmetrize,
                          weighted=weighted, threads=threads)
    return Graph.er(1 << spec.scale, spec.edge_factor, spec.seed, symmetrize=symmetrize, weighted=weighted,
                    threads=threads)


class Union:
    """Disjoint union of host graphs (copied into one CSR)."""

    def __init__(self, graphs: Sequence[Graph]):
        sizes = np.array([G.num_vertices for G in graphs], dtype=np.int64)
        edges = np.array([G.num_edges for G in graphs], dtype=np.int64)
        self.bases = np.concatenate([[0], np.cumsum(sizes)])[:-1]
        self.sizes = sizes
        V, E = int(sizes.sum()), int(edges.sum())
        if V >= 2**32 - 1 or E >= 2**32 - 16:
            raise ValueError("batch too large for 32-bit ids / offsets")
        ro = np.empty(V + 1, dtype=np.uint64)
        col = np.empty(E, dtype=np.uint32)
        weighted = all(G.weights is not None for G in graphs)
        w = np.empty(E, dtype=np.uint32) if weighted else None
        eoff = 0
        for G, base in zip(graphs, self.bases):
            n, m = G.num_vertices, G.num_edges
            ro[base:base + n] = G.row_offsets[:-1] + np.uint64(eoff)
            col[eoff:eoff + m] = G.col_indices + np.uint32(base)
            if weighted:
                w[eoff:eoff + m] = G.weights
            eoff += m
        ro[V] = E
        self.graph = Graph.from_csr(ro, col, w)

    def split(self, arr: np.ndarray) -> List[np.ndarray]:
        return [arr[b:b + n] for b, n in zip(self.bases, self.sizes)]

    def split_labels(self, labels: np.ndarray) -> List[np.ndarray]:
        return [(part - np.uint32(b)).astype(np.uint32) for part, b in zip(self.split(labels), self.bases)]


def run_plain_graphs(graphs_cc: Sequence[Graph], graphs_pr: Sequence[Graph], pr_iters: int = 20, device: int = 0,
                     num_memory: int = 1, concurrent: bool = False):
    """One ctx per graph (the unbatched path).  concurrent=False runs the
    algorithms graph after graph, each run waited for; concurrent=True
    initialises every ctx, then queues all runs at once (GRD_RUN_ASYNC, one
    stream per ctx, so small graphs' runs overlap on the GPU) and waits for
    them.  Returns (labels, ranks, seconds)."""
    import time
    ctxs = [(Context(Gc, None, num_memory, device), Context(Gp, None, num_memory, device))
            for Gc, Gp in zip(graphs_cc, graphs_pr)]
    for cc, pr in ctxs:
        cc.set_algo(GRD_CC)
        pr.set_algo(GRD_PR_PULL, max_rounds=pr_iters, tolerance=0.0)
    labels, ranks = [], []
    t0 = time.perf_counter()
    if concurrent:
        for cc, pr in ctxs:
            cc.init()
            pr.init()
        for cc, pr in ctxs:
            cc.run(wait=False)
            pr.run(wait=False)
        for cc, pr in ctxs:
            cc.wait()
            pr.wait()
    else:
        for cc, pr in ctxs:
            cc.init()
            cc.run()
            pr.init()
            pr.run()
        for cc, pr in ctxs:
            cc.synchronize()
    secs = time.perf_counter() - t0
    for cc, pr in ctxs:
        labels.append(cc.read_props())
        ranks.append(pr.read_ranks())
        cc.close()
        pr.close()
    return labels, ranks, secs
