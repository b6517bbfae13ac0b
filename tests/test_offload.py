"""Offload decision per round (NDPEngine, include/offload_engine/NDPEngine.hpp:
10-51) and the NO_OFFLOAD round (src/GraphAlgorithm.cpp:426-474, 582-637):
oracle checks on the CPU, GPU parity through the C ABI.

NO_OFFLOAD rounds ship each frontier vertex's adjacency to the compute
partition, which applies the algorithm's own update to its vertex_updates.
Min-aggregated results (CC, SSSP) and round counts equal those of the
reference's all-NDP_OFFLOAD run bit for bit; PageRank equals it up to float
summation order.
"""
import numpy as np
import pytest

import grudon_gb300 as g
from oracle import ffi as O

OFFLOADS = [O.ORC_OFFLOAD_ENGINE, O.ORC_OFFLOAD_NONE]


def _levels(dist):
    d = dist[dist != 0xFFFFFFFF]
    return np.bincount(d.astype(np.int64))


@pytest.mark.parametrize("num_memory", [1, 3])
def test_oracle_no_offload_matches_ndp(num_memory):
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    L = O.Layout(ro, ci, w, part, num_memory)
    for a in (O.ORC_CC, O.ORC_SSSP_HOP, O.ORC_SSSP_W):
        ndp = L.run(a)
        for off in OFFLOADS:
            r = L.run(a, offload=off)
            np.testing.assert_array_equal(r["props"], ndp["props"])
            np.testing.assert_array_equal(r["updates"], ndp["updates"])
            for k in ("rounds", "converged", "edges_scanned"):
                assert r["stats"][k] == ndp["stats"][k], k
        assert L.run(a, offload=O.ORC_OFFLOAD_NONE)["stats"]["no_offload_rounds"] == ndp["stats"]["rounds"]
    ndp = L.run(O.ORC_PR_DELTA)
    for off in OFFLOADS:
        r = L.run(O.ORC_PR_DELTA, offload=off)
        np.testing.assert_allclose(r["ranks"], ndp["ranks"], rtol=1e-4, atol=2e-5)
    # and against the textbook oracles
    np.testing.assert_array_equal(L.run(O.ORC_CC, offload=O.ORC_OFFLOAD_NONE)["props"], O.cc_union_find(ro, ci))
    np.testing.assert_array_equal(L.run(O.ORC_SSSP_W, offload=O.ORC_OFFLOAD_NONE)["props"],
                                  O.dijkstra(ro, ci, w, 0))


def test_oracle_no_offload_bytes_by_hand():
    """Path 0->1->2->3 (+ 0->2), one memory partition, SSSP hop from 0,
    every round NO_OFFLOAD.  Per round: the forward sync (one 64-bit word,
    counted x8 by the reference, plus 4 B per frontier value) and one
    adjacency message per frontier vertex of 1 + out-degree gids, counted at
    the send and at the receive."""
    ro = [0, 2, 3, 4, 4]
    ci = [1, 2, 2, 3]
    r = O.run(O.ORC_SSSP_HOP, ro, ci, offload=O.ORC_OFFLOAD_NONE)
    assert list(r["props"]) == [0, 1, 1, 2]
    # rounds: {0} (deg 2) -> {1, 2} (deg 1, 1) -> {3} (deg 0) -> empty
    fronts = [[2], [1, 1], [0]]
    bytes_true = sum(8 + 4 * len(f) + 4 * sum(1 + d for d in f) for f in fronts)
    bytes_ref = sum(64 + 4 * len(f) + 8 * sum(1 + d for d in f) for f in fronts)
    st = r["stats"]
    assert st["rounds"] == 3 and st["no_offload_rounds"] == 3
    assert st["bytes_synced"] == bytes_true
    assert st["reference_bytes_moved"] == bytes_ref
    # weighted: the message also carries one weight per edge
    rw = O.run(O.ORC_SSSP_W, ro, ci, [5, 1, 1, 1], offload=O.ORC_OFFLOAD_NONE)
    assert list(rw["props"]) == [0, 5, 1, 2]
    # rounds: {0} -> {1, 2} (1 at 5, 2 at 1) -> {3} -> empty
    assert rw["stats"]["bytes_synced"] == sum(8 + 4 * len(f) + 4 * sum(1 + 2 * d for d in f) for f in fronts)


def test_oracle_ndp_engine_threshold():
    """NDPEngine with one compute partition: NO_OFFLOAD exactly in the rounds
    whose frontier holds 1..V/20 vertices (coverage always holds, and the
    busiest partition never falls below the mean)."""
    G = g.Graph.rmat(12, 8, symmetrize=True)
    ro, ci = G.row_offsets, G.col_indices
    V = G.num_vertices
    for M in (1, 4):
        part = G.partition_edge_balanced(M) if M > 1 else None
        r = O.run(O.ORC_SSSP_HOP, ro, ci, mirror=part, num_memory=M, offload=O.ORC_OFFLOAD_ENGINE)
        # round k's frontier is BFS level k
        sizes = _levels(r["props"])
        assert r["stats"]["rounds"] == len(sizes)
        assert r["stats"]["no_offload_rounds"] == int(np.sum((sizes > 0) & (sizes <= V // 20)))
        assert 0 < r["stats"]["no_offload_rounds"] < r["stats"]["rounds"]


def test_threaded_oracle_no_offload():
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(3)
    for a in (O.ORC_CC, O.ORC_SSSP_W):
        s = O.run(a, ro, ci, w, mirror=part, num_memory=3, offload=O.ORC_OFFLOAD_ENGINE)
        t = O.run(a, ro, ci, w, mirror=part, num_memory=3, offload=O.ORC_OFFLOAD_ENGINE, threads=4)
        np.testing.assert_array_equal(s["props"], t["props"])
        assert s["stats"] == t["stats"]


# ---------------------------------------------------------------- GPU ----
GPU_ALGOS = [(g.GRD_CC, O.ORC_CC), (g.GRD_SSSP_HOP, O.ORC_SSSP_HOP), (g.GRD_SSSP_W, O.ORC_SSSP_W)]
GRAPHS = {
    "rmat13_sym": lambda: g.Graph.rmat(13, 8, symmetrize=True, weighted=True),
    "rmat13_dir": lambda: g.Graph.rmat(13, 16, weighted=True),
    "grid60": lambda: g.Graph.grid(60, seed=3),
}
GPU_OFFLOADS = [(g.GRD_OFFLOAD_ENGINE, O.ORC_OFFLOAD_ENGINE), (g.GRD_OFFLOAD_NONE, O.ORC_OFFLOAD_NONE)]


@pytest.mark.gpu
@pytest.mark.parametrize("host_loop", [False, True], ids=["device-loop", "host-loop"])
@pytest.mark.parametrize("offload", GPU_OFFLOADS, ids=["engine", "none"])
@pytest.mark.parametrize("num_memory", [1, 3])
@pytest.mark.parametrize("name", list(GRAPHS))
def test_gpu_no_offload_bit_exact(gpu, name, num_memory, offload, host_loop):
    G = GRAPHS[name]()
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    L = O.Layout(ro, ci, w, part, num_memory)
    with g.Context(G, part, num_memory=num_memory) as ctx:
        for algo, oalgo in GPU_ALGOS:
            ctx.set_algo(algo, offload=offload[0])
            ctx.init()
            st = ctx.run(host_loop=host_loop)
            ref = L.run(oalgo, offload=offload[1])
            np.testing.assert_array_equal(ctx.read_props(), ref["props"])
            np.testing.assert_array_equal(ctx.read_updates(), ref["updates"])
            for k in ("rounds", "converged", "edges_scanned", "bytes_synced", "reference_bytes_moved",
                      "no_offload_rounds"):
                assert st[k] == ref["stats"][k], k
            assert st["device_loop"] == (0 if host_loop else 1)
            assert st["pull_rounds"] == 0 and st["push_rounds"] == st["rounds"]


@pytest.mark.gpu
@pytest.mark.parametrize("offload", GPU_OFFLOADS, ids=["engine", "none"])
def test_gpu_no_offload_pagerank(gpu, offload):
    G = g.Graph.rmat(13, 8)
    ro, ci = G.row_offsets, G.col_indices
    part = G.partition_edge_balanced(2)
    ref = O.run(O.ORC_PR_DELTA, ro, ci, mirror=part, num_memory=2, offload=offload[1])
    with g.Context(G, part, num_memory=2) as ctx:
        ctx.set_algo(g.GRD_PR_DELTA, offload=offload[0])
        ctx.init()
        st = ctx.run()
        np.testing.assert_allclose(ctx.read_ranks(), ref["ranks"], rtol=1e-4, atol=2e-5)
        assert abs(st["rounds"] - ref["stats"]["rounds"]) <= 1
        assert st["no_offload_rounds"] > 0


@pytest.mark.gpu
def test_gpu_no_offload_with_profiling_round_log(gpu):
    """Profiled host-loop rounds record the NO_OFFLOAD mode; the engine mixes
    it with the fixed rule's NDP rounds."""
    G = g.Graph.rmat(14, 8, symmetrize=True, weighted=True)
    V = G.num_vertices
    with g.Context(G, G.partition_edge_balanced(2), num_memory=2) as ctx:
        ctx.set_profiling(True)
        ctx.set_algo(g.GRD_SSSP_HOP, offload=g.GRD_OFFLOAD_ENGINE)
        ctx.init()
        st = ctx.run()
        log = ctx.round_log()
        assert len(log) == st["rounds"]
        for r in log:
            small = 0 < r["frontier_in"] <= V // 20
            assert (r["mode"] == g.GRD_ROUND_NO_OFFLOAD) == small
        assert sum(r["mode"] == g.GRD_ROUND_NO_OFFLOAD for r in log) == st["no_offload_rounds"] > 0
        ref = O.run(O.ORC_SSSP_HOP, G.row_offsets, G.col_indices, mirror=G.partition_edge_balanced(2),
                    num_memory=2, offload=O.ORC_OFFLOAD_ENGINE)
        np.testing.assert_array_equal(ctx.read_props(), ref["props"])
        assert st["bytes_synced"] == ref["stats"]["bytes_synced"]


@pytest.mark.gpu
def test_gpu_offload_rejected_for_pull_pagerank(gpu):
    G = g.Graph.rmat(10, 8)
    with g.Context(G) as ctx:
        with pytest.raises(g.GrdError):
            ctx.set_algo(g.GRD_PR_PULL, offload=g.GRD_OFFLOAD_ENGINE)
        with pytest.raises(g.GrdError):
            ctx.set_algo(g.GRD_CC, offload=7)


@pytest.mark.gpu
def test_gpu_no_offload_multi_source_batch(gpu):
    """Many SSSP sources (a batch of graph copies) with the engine: same
    distances as the all-NDP run."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    srcs = np.array([0, 17, 999, 4000], dtype=np.uint32)
    out = []
    with g.Context(G, G.partition_edge_balanced(3), num_memory=3) as ctx:
        for off in (g.GRD_OFFLOAD_NDP, g.GRD_OFFLOAD_ENGINE, g.GRD_OFFLOAD_NONE):
            ctx.set_algo(g.GRD_SSSP_W, offload=off)
            ctx.init_sources(srcs)
            st = ctx.run()
            out.append((ctx.read_props(), st["rounds"], st["edges_scanned"]))
    for p, r, e in out[1:]:
        np.testing.assert_array_equal(p, out[0][0])
        assert (r, e) == out[0][1:]


@pytest.mark.gpu
@pytest.mark.parametrize("algo", [g.GRD_CC, g.GRD_SSSP_W])
def test_gpu_no_offload_sees_values_aggregated_between_rounds(gpu, algo):
    """grd_aggregate_values before a run lists gids for the next update;
    NO_OFFLOAD rounds (which append to the same list) keep them."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    gids = np.array([5, 77, 5, 1000], dtype=np.uint32)
    vals = np.array([0, 3, 2, 1], dtype=np.uint32)
    outs = []
    with g.Context(G, G.partition_edge_balanced(3), num_memory=3) as ctx:
        for off in (g.GRD_OFFLOAD_NDP, g.GRD_OFFLOAD_ENGINE, g.GRD_OFFLOAD_NONE):
            for host_loop in (True, False):
                ctx.set_algo(algo, offload=off, frontier_format=g.GRD_FMT_LIST)
                ctx.init()
                rc = ctx._lib.grd_aggregate_values(ctx._ctx, gids.ctypes.data_as(g._ffi.u32p),
                                                   vals.ctypes.data_as(g._ffi.u32p), len(gids))
                assert rc == 0
                st = ctx.run(host_loop=host_loop)
                outs.append((ctx.read_props(), ctx.read_updates(), st["rounds"]))
    for p, u, r in outs[1:]:
        np.testing.assert_array_equal(p, outs[0][0])
        np.testing.assert_array_equal(u, outs[0][1])
        assert r == outs[0][2]


@pytest.mark.gpu
def test_gpu_no_offload_cli(gpu, tmp_path):
    """The flag-compatible driver accepts --offload and prints the same
    checksum as the default schedule."""
    import subprocess
    from pathlib import Path
    cli = Path(g.__file__).resolve().parent / "_build" / "grudon"
    if not cli.exists():
        pytest.skip("driver not built")
    G = g.Graph.rmat(11, 8, symmetrize=True)
    path = tmp_path / "g.gr"
    G.write_gr(str(path))
    outs = []
    for extra in ([], ["--offload", "engine"], ["--offload", "none"]):
        r = subprocess.run([str(cli), "-g", str(path), "-c", "1", "-m", "2", "-a", "cc", *extra],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append([l for l in r.stdout.splitlines() if l.startswith(("CHECKSUM", "STAT"))
                     and "TotalBytesMoved" not in l])
    assert outs[1] == outs[0] and outs[2] == outs[0]
