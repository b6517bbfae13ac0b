"""grd_sssp_multi: distances from up to 64 sources at once over one resident
CSR, each lane against the textbook single-source oracles (Dijkstra for
weighted SSSP, BFS for hop counts), bit for bit."""
import numpy as np
import pytest

import grudon_gb300 as g
from grudon_gb300 import _ffi
from oracle import ffi as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("num_memory", [1, 3])
def test_multi_source_weighted_equals_dijkstra(gpu, num_memory):
    G = g.Graph.rmat(13, 16, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    rng = np.random.default_rng(11)
    sources = rng.integers(0, G.num_vertices, 64)
    sources[:3] = [0, 0, int(sources[5])]  # repeats are fine
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    with g.Context(G, part, num_memory=num_memory) as ctx:
        ctx.set_algo(g.GRD_SSSP_W)
        ctx.init()
        dist, st = ctx.sssp_multi(sources)
        assert dist.shape == (64, G.num_vertices) and st["converged"] == 1
        for l, s in enumerate(sources):
            np.testing.assert_array_equal(dist[l], O.dijkstra(ro, ci, w, int(s)))
        # a second call reuses the arrays and starts from scratch
        dist2, _ = ctx.sssp_multi(sources[:5])
        np.testing.assert_array_equal(dist2, dist[:5])


def test_multi_source_hops_equal_bfs_and_the_single_source_run(gpu):
    G = g.Graph.grid(40, weighted=False)
    ro, ci = G.row_offsets, G.col_indices
    sources = [0, 799, 1599, 17]
    with g.Context(G, G.partition_edge_balanced(2), num_memory=2) as ctx:
        ctx.set_algo(g.GRD_SSSP_HOP)
        ctx.init()
        dist, st = ctx.sssp_multi(sources)
        for l, s in enumerate(sources):
            np.testing.assert_array_equal(dist[l], O.bfs(ro, ci, s))
        ctx.set_algo(g.GRD_SSSP_HOP, source=799)
        ctx.init()
        ctx.run()
        np.testing.assert_array_equal(ctx.read_props(), dist[1])


def test_multi_source_refuses_bad_arguments(gpu):
    G = g.Graph.rmat(8, 4, weighted=True)
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        with pytest.raises(g.GrdError):
            ctx.sssp_multi([0])
        ctx.set_algo(g.GRD_SSSP_W)
        ctx.init()
        with pytest.raises(g.GrdError):
            ctx.sssp_multi(list(range(65)))
        with pytest.raises(g.GrdError):
            ctx.sssp_multi([G.num_vertices])
