"""Batched workloads: disjoint-union layout (CPU) and batched runs against
per-graph oracles (GPU)."""
import numpy as np
import pytest

import grudon_gb300 as g
from grudon_gb300 import batch as B
from oracle import ffi as O


def test_batch_spec_distribution():
    spec = B.batch_spec(512)
    assert spec == B.batch_spec(512)  # seeded
    scales = np.array([s.scale for s in spec])
    assert scales.min() >= 10 and scales.max() <= 18
    assert np.mean(scales <= 13) > 0.5  # log-uniform favours small scales
    assert {s.edge_factor for s in spec} == {4, 8, 16, 32}
    assert sum(s.kind == "rmat" for s in spec) == 256
    a = np.array([s.a for s in spec])
    assert a.min() >= 0.45 and a.max() <= 0.65
    b = spec[0].abc
    assert abs(sum(b) + B.ER_D - 1.0) < 1e-12 and b[1] == b[2]


def test_union_layout_and_split():
    graphs = [g.Graph.rmat(6, 4, weighted=True), g.Graph.er(50, 3, seed=2, weighted=True), g.Graph.grid(4)]
    U = B.Union(graphs)
    G = U.graph
    assert G.num_vertices == sum(x.num_vertices for x in graphs)
    assert G.num_edges == sum(x.num_edges for x in graphs)
    for x, base, part_ro in zip(graphs, U.bases, U.split(np.diff(G.row_offsets.astype(np.int64)))):
        np.testing.assert_array_equal(part_ro, np.diff(x.row_offsets.astype(np.int64)))
        lo = int(G.row_offsets[base])
        np.testing.assert_array_equal(G.col_indices[lo:lo + x.num_edges] - base, x.col_indices)
        np.testing.assert_array_equal(G.weights[lo:lo + x.num_edges], x.weights)
    # CC labels of the union restrict to each graph's own labels
    S = [g.Graph.rmat(7, 4, symmetrize=True), g.Graph.er(100, 2, seed=5, symmetrize=True)]
    US = B.Union(S)
    lab = O.cc_union_find(US.graph.row_offsets, US.graph.col_indices)
    for part, x in zip(US.split_labels(lab), S):
        np.testing.assert_array_equal(part, O.cc_union_find(x.row_offsets, x.col_indices))


@pytest.mark.gpu
def test_batched_cc_and_pagerank_match_per_graph(gpu):
    spec = B.batch_spec(12, seed=3, lo=6, hi=11)
    sym = [B.make_graph(s, symmetrize=True) for s in spec]
    dirg = [B.make_graph(s) for s in spec]
    Uc, Up = B.Union(sym), B.Union(dirg)
    with g.Context(Uc.graph) as c:
        c.set_algo(g.GRD_CC)
        c.init()
        c.run()
        for part, x in zip(Uc.split_labels(c.read_props()), sym):
            np.testing.assert_array_equal(part, O.cc_union_find(x.row_offsets, x.col_indices))
    with g.Context(Up.graph) as c:
        c.set_algo(g.GRD_PR_PULL, max_rounds=20, tolerance=0.0)
        c.init()
        st = c.run()
        assert st["rounds"] == 20
        for part, x in zip(Up.split(c.read_ranks()), dirg):
            ref, _, _ = O.pr_jacobi_fp64(x.row_offsets, x.col_indices, iters=20)
            rel = np.abs(part - ref) / np.maximum(ref, 1e-30)
            assert np.max(np.where((part == 0) & (ref == 0), 0, rel)) <= 1e-5


@pytest.mark.gpu
def test_multi_source_sssp_union(gpu):
    G = g.Graph.rmat(12, 8, weighted=True)
    rng = np.random.default_rng(1)
    sources = rng.integers(0, G.num_vertices, 6)
    U = B.Union([G] * len(sources))
    with g.Context(U.graph, U.graph.partition_edge_balanced(3), 3) as c:
        c.set_algo(g.GRD_SSSP_W)
        c.init_sources(U.bases + sources)
        c.run()
        for part, s in zip(U.split(c.read_props()), sources):
            np.testing.assert_array_equal(part, O.dijkstra(G.row_offsets, G.col_indices, G.weights, int(s)))


@pytest.mark.gpu
def test_autotuner_candidates_agree(gpu):
    from grudon_gb300 import autotune
    G = g.Graph.rmat(14, 8, symmetrize=True)
    res = autotune.tune(G, g.GRD_CC, lambda c: c.init(),
                        space=[autotune.Candidate(1, 8, 0), autotune.Candidate(3, 128, 2)], reps=1)
    assert len(res.table) == 2 and res.best_ms > 0
    outs = []
    for cand in (autotune.Candidate(1, 8, 0), autotune.Candidate(3, 128, 2)):
        part = G.partition_edge_balanced(cand.num_memory) if cand.num_memory > 1 else None
        with g.Context(G, part, cand.num_memory) as c:
            c.set_algo(g.GRD_CC, **cand.params())
            c.init()
            c.run()
            outs.append(c.read_props())
    np.testing.assert_array_equal(outs[0], outs[1])
