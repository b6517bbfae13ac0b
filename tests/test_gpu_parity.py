"""GPU parity: the CUDA path (through the C ABI) against the oracle.

CC and SSSP are compared bit-exactly (labels, distances, round counts, wire
statistics); delta PageRank within an absolute 2e-5 + relative 1e-4 bound on
pr_vals (float atomics make the per-vertex summation order nondeterministic,
exactly as the reference's concurrent atomicAdd does).
"""
import numpy as np
import pytest

import grudon_gb300 as g
from oracle import ffi as O

pytestmark = pytest.mark.gpu

ALGOS = [(g.GRD_CC, O.ORC_CC), (g.GRD_SSSP_HOP, O.ORC_SSSP_HOP), (g.GRD_SSSP_W, O.ORC_SSSP_W)]


GRAPHS = {
    "rmat12_sym": lambda: g.Graph.rmat(12, 8, symmetrize=True, weighted=True),
    "rmat13_dir": lambda: g.Graph.rmat(13, 16, weighted=True),
    "er4k": lambda: g.Graph.er(4000, 4, seed=7, symmetrize=True, weighted=True),
    "grid40": lambda: g.Graph.grid(40, seed=3),
}


FORMATS = [g.GRD_FMT_AUTO, g.GRD_FMT_BITVEC, g.GRD_FMT_LIST]
# (direction, sync format): every round mode forced, and the fixed heuristic
# choosing per round.
MODES = [(g.GRD_DIR_PUSH, g.GRD_FMT_LIST), (g.GRD_DIR_PUSH, g.GRD_FMT_BITVEC), (g.GRD_DIR_PULL, g.GRD_FMT_BITVEC),
         (g.GRD_DIR_PULL, g.GRD_FMT_LIST), (g.GRD_DIR_AUTO, g.GRD_FMT_AUTO)]
MODE_IDS = ["push-list", "push-bitvec", "pull-bitvec", "pull-list", "auto"]


@pytest.mark.parametrize("num_memory", [1, 3])
@pytest.mark.parametrize("name", list(GRAPHS))
@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
def test_min_algorithms_bit_exact(gpu, name, num_memory, mode):
    G = GRAPHS[name]()
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    direction, fmt = mode
    with g.Context(G, part, num_memory=num_memory) as ctx:
        for algo, oalgo in ALGOS:
            ctx.set_algo(algo, direction=direction, frontier_format=fmt)
            ctx.init()
            st = ctx.run()
            ref = O.run(oalgo, ro, ci, w, mirror=part, num_memory=num_memory)
            np.testing.assert_array_equal(ctx.read_props(), ref["props"])
            np.testing.assert_array_equal(ctx.read_updates(), ref["updates"])
            assert st["rounds"] == ref["stats"]["rounds"]
            assert st["converged"] == 1
            if direction == g.GRD_DIR_PUSH:
                assert st["edges_scanned"] == ref["stats"]["edges_scanned"]
                assert st["pull_rounds"] == 0
            if direction == g.GRD_DIR_PULL:
                assert st["push_rounds"] == 0 and st["edges_scanned"] == st["rounds"] * G.num_edges
            assert st["bytes_synced"] == ref["stats"]["bytes_synced"]
            assert st["reference_bytes_moved"] == ref["stats"]["reference_bytes_moved"]


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
def test_device_loop_matches_host_loop(gpu, mode):
    """One CUDA-graph launch (device-side policy + switch + while) gives the
    same results and statistics as the host-driven loop."""
    G = g.Graph.rmat(13, 8, symmetrize=True, weighted=True)
    part = G.partition_edge_balanced(3)
    with g.Context(G, part, num_memory=3) as ctx:
        for algo in (g.GRD_CC, g.GRD_SSSP_HOP, g.GRD_SSSP_W, g.GRD_PR_DELTA):
            ctx.set_algo(algo, direction=mode[0], frontier_format=mode[1])
            ctx.init()
            hs = ctx.run(host_loop=True)
            hp, hr = ctx.read_props(), ctx.read_ranks()
            ctx.init()
            ds = ctx.run()
            assert hs["device_loop"] == 0 and ds["device_loop"] == 1
            if algo == g.GRD_PR_DELTA:  # fixed-order sums: the same ranks bit for bit
                np.testing.assert_array_equal(ctx.read_ranks(), hr)
            np.testing.assert_array_equal(ctx.read_props(), hp)
            for k in ("rounds", "converged", "edges_scanned", "bytes_synced", "reference_bytes_moved",
                      "push_rounds", "pull_rounds", "actives_total", "push_actives"):
                assert ds[k] == hs[k], k
            # the device loop adds its policy and round-end kernels each round,
            # except for small rounds run back to back inside one kernel
            assert ds["kernel_launches"] <= hs["kernel_launches"] + 2 * ds["rounds"]


def test_device_loop_respects_round_cap(gpu):
    G = g.Graph.grid(30)
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_SSSP_HOP, max_rounds=5)
        ctx.init()
        st = ctx.run()
        assert st["device_loop"] == 1 and st["rounds"] == 5 and st["converged"] == 0
        ref = O.run(O.ORC_SSSP_HOP, G.row_offsets, G.col_indices, max_rounds=5)
        np.testing.assert_array_equal(ctx.read_props(), ref["props"])


def test_round_log_modes_follow_policy(gpu):
    """Forced formats run every round in that mode; the fixed rule mixes
    bitvector rounds (large frontiers) and list rounds (small ones)."""
    G = g.Graph.rmat(14, 8, symmetrize=True, weighted=True)
    expect = {(g.GRD_DIR_PUSH, g.GRD_FMT_LIST): {g.GRD_ROUND_PUSH_LIST},
              (g.GRD_DIR_PUSH, g.GRD_FMT_BITVEC): {g.GRD_ROUND_PUSH_BITVEC},
              (g.GRD_DIR_PULL, g.GRD_FMT_LIST): {g.GRD_ROUND_PULL_LIST},
              (g.GRD_DIR_PULL, g.GRD_FMT_BITVEC): {g.GRD_ROUND_PULL_BITVEC}}
    with g.Context(G, G.partition_edge_balanced(2), num_memory=2) as ctx:
        ctx.set_profiling(True)
        for (d, f), modes in expect.items():
            ctx.set_algo(g.GRD_CC, direction=d, frontier_format=f)
            ctx.init()
            ctx.run()
            assert {r["mode"] for r in ctx.round_log()} == modes
    # a fresh context has no in-edge view, so the fixed rule only pushes
    with g.Context(G, G.partition_edge_balanced(2), num_memory=2) as ctx:
        ctx.set_profiling(True)
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        ctx.run()
        log = ctx.round_log()
        tile = 8192  # slots per partition are padded to whole compaction tiles
        S = sum(-(-(no + npx) // tile) * tile for no, npx, _ in (ctx.layout_info(p) for p in range(2)))
        for r in log:
            big = r["frontier_in"] * 8 >= S or r["frontier_edges_in"] * 8 >= G.num_edges
            assert r["mode"] == (g.GRD_ROUND_PUSH_BITVEC if big else g.GRD_ROUND_PUSH_LIST)
        assert {r["mode"] for r in log} == {g.GRD_ROUND_PUSH_BITVEC, g.GRD_ROUND_PUSH_LIST}


@pytest.mark.parametrize("algo", [g.GRD_CC, g.GRD_SSSP_W])
def test_values_aggregated_between_rounds_reach_list_rounds(gpu, algo):
    """grd_aggregate_values before a run: list rounds see the same updated
    gids as bitvector rounds."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    gids = np.array([5, 77, 5, 1000], dtype=np.uint32)
    vals = np.array([0, 3, 2, 1], dtype=np.uint32)
    outs = []
    with g.Context(G, G.partition_edge_balanced(3), num_memory=3) as ctx:
        for fmt in (g.GRD_FMT_BITVEC, g.GRD_FMT_LIST):
            for host_loop in (True, False):
                ctx.set_algo(algo, frontier_format=fmt)
                ctx.init()
                rc = ctx._lib.grd_aggregate_values(ctx._ctx, gids.ctypes.data_as(g._ffi.u32p),
                                                   vals.ctypes.data_as(g._ffi.u32p), len(gids))
                assert rc == 0
                ctx.run(host_loop=host_loop)
                outs.append((ctx.read_props(), ctx.read_updates()))
    for p, u in outs[1:]:
        np.testing.assert_array_equal(p, outs[0][0])
        np.testing.assert_array_equal(u, outs[0][1])


@pytest.mark.parametrize("num_memory", [1, 3])
def test_stage_api_matches_oracle_round_by_round(gpu, num_memory):
    G = g.Graph.rmat(11, 8, symmetrize=True, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    with g.Context(G, part, num_memory=num_memory) as ctx:
        for algo, oalgo in ALGOS:
            ctx.set_algo(algo)
            ctx.init()
            r = 0
            while True:
                f = ctx.round()
                r += 1
                ref = O.run(oalgo, ro, ci, w, mirror=part, num_memory=num_memory, max_rounds=r)
                np.testing.assert_array_equal(ctx.read_props(), ref["props"])
                np.testing.assert_array_equal(ctx.read_updates(), ref["updates"])
                if f == 0:
                    break
            assert r == ref["stats"]["rounds"]


@pytest.mark.parametrize("num_memory", [1, 3])
@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
def test_pr_delta_bit_exact_to_oracle(gpu, num_memory, mode):
    """Delta PageRank sums every destination's frontier contributions in one
    fixed order (in-list chunks of 32, a halving tree per chunk) and
    aggregates partitions in ascending order, as the oracle does: ranks,
    round counts and byte statistics equal the oracle's in every round mode."""
    G = g.Graph.rmat(14, 16)
    ro, ci = G.row_offsets, G.col_indices
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    with g.Context(G, part, num_memory=num_memory) as ctx:
        ctx.set_algo(g.GRD_PR_DELTA, direction=mode[0], frontier_format=mode[1])
        if num_memory == 1:  # in-lists above 1024 edges take the chunked grid-wide path
            assert len(ctx.read_layout("in_hubs")) > 0
        ctx.init()
        st = ctx.run()
        ref = O.run(O.ORC_PR_DELTA, ro, ci, mirror=part, num_memory=num_memory)
        np.testing.assert_array_equal(ctx.read_ranks(), ref["ranks"])
        assert st["rounds"] == ref["stats"]["rounds"]
        assert st["bytes_synced"] == ref["stats"]["bytes_synced"]


def test_pr_delta_identical_under_every_policy(gpu):
    """The four forced round modes, the fixed rule and the learned policy
    (shipped model and random models) give bit-identical delta-PageRank
    ranks, on a power-law graph and a grid."""
    from grudon_gb300 import policy as P
    from test_policy import random_model
    models = [random_model(seed) for seed in (1, 2)]
    if P.MODEL_FILE.exists():
        models.append(P.load_model())
    for G in (g.Graph.rmat(15, 16), g.Graph.grid(128)):
        part = G.partition_edge_balanced(3)
        with g.Context(G, part, num_memory=3) as ctx:
            outs = []
            for kw in [dict(direction=d, frontier_format=f) for d, f in P.FORCED] + [{}]:
                ctx.set_algo(g.GRD_PR_DELTA, **kw)
                ctx.init()
                ctx.run()
                outs.append(ctx.read_ranks())
            for m in models:
                ctx.set_algo(g.GRD_PR_DELTA, policy=g.GRD_POLICY_LEARNED)
                ctx.set_policy(m)
                ctx.init()
                ctx.run()
                outs.append(ctx.read_ranks())
            for o in outs[1:]:
                np.testing.assert_array_equal(o, outs[0])


def test_cc_sssp_full_size_properties(gpu):
    """RMAT-18 symmetric: CC against union-find, SSSP against BFS / Dijkstra."""
    G = g.Graph.rmat(18, 16, symmetrize=True, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(3)
    with g.Context(G, part, num_memory=3) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        ctx.run()
        np.testing.assert_array_equal(ctx.read_props(), O.cc_union_find(ro, ci))
        ctx.set_algo(g.GRD_SSSP_HOP)
        ctx.init()
        ctx.run()
        np.testing.assert_array_equal(ctx.read_props(), O.bfs(ro, ci, 0))
        ctx.set_algo(g.GRD_SSSP_W)
        ctx.init()
        ctx.run()
        np.testing.assert_array_equal(ctx.read_props(), O.dijkstra(ro, ci, w, 0))


def test_edge_cases(gpu):
    # single vertex, no edges
    G = g.Graph.from_csr([0, 0], [])
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        st = ctx.run()
        assert st["rounds"] == 1 and list(ctx.read_props()) == [0]
    # isolated vertices + one edge; unreachable SSSP stays UINT32_MAX
    G = g.Graph.from_edges(5, [1], [3], [7])
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_SSSP_W, source=1)
        ctx.init()
        ctx.run()
        assert list(ctx.read_props()) == [0xFFFFFFFF, 0, 0xFFFFFFFF, 7, 0xFFFFFFFF]
    # round cap
    G = g.Graph.grid(20)
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_SSSP_HOP, max_rounds=3)
        ctx.init()
        st = ctx.run()
        assert st["rounds"] == 3 and st["converged"] == 0
        ctx.init()
        with pytest.raises(g.GrdError):
            ctx.run(strict=True)


def _max_rel_err(got, exp):
    got = np.asarray(got, dtype=np.float64)
    both_zero = (got == 0) & (exp == 0)
    rel = np.abs(got - exp) / np.maximum(np.abs(exp), 1e-300)
    return float(np.max(np.where(both_zero, 0.0, rel)))


@pytest.mark.parametrize("num_memory", [1, 3])
def test_pr_pull_vs_fp64_oracle(gpu, num_memory):
    """FP32 Kahan pull PageRank within max relative error 1e-5 of FP64 Jacobi
    run for the same number of iterations (the config-3 accuracy bar)."""
    G = g.Graph.rmat(15, 16)
    ro, ci = G.row_offsets, G.col_indices
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    with g.Context(G, part, num_memory=num_memory) as ctx:
        ctx.set_algo(g.GRD_PR_PULL, max_rounds=40, tolerance=0.0)
        ctx.init()
        st = ctx.run()
        assert st["rounds"] == 40 and st["converged"] == 0
        ref, it, res = O.pr_jacobi_fp64(ro, ci, iters=40)
        assert it == 40
        assert _max_rel_err(ctx.read_ranks(), ref) <= 1e-5
        assert abs(st["last_residual"] - res) <= 1e-3 * res + 1e-12
        assert st["edges_scanned"] == 40 * G.num_edges


def test_pr_pull_rmat20_exact_degree_hot_cut(gpu):
    """RMAT-20: the 32 768-source cap of the shared-memory hot set falls
    inside an out-degree histogram bucket (degrees 64-79), so the set is cut
    at an exact degree inside it (about 32 100 hot sources instead of the
    bucket boundary's 25 300).  A hot source read from the wrong place would
    show in the ranks: they stay within 1e-5 of FP64 Jacobi, and two runs
    agree bit for bit."""
    G = g.Graph.rmat(20, 16)
    ro, ci = G.row_offsets, G.col_indices
    deg = np.diff(ro.astype(np.int64))
    assert 25_000 < int((deg >= 80).sum()) <= 32_768 < int((deg >= 64).sum())  # the cap falls in [64, 80)
    with g.Context(G, G.partition_edge_balanced(3), num_memory=3) as ctx:
        ctx.set_algo(g.GRD_PR_PULL, max_rounds=30, tolerance=0.0)
        runs = []
        for _ in range(2):
            ctx.init()
            st = ctx.run()
            assert st["rounds"] == 30
            runs.append(ctx.read_ranks())
    np.testing.assert_array_equal(runs[0], runs[1])
    ref, it, _ = O.pr_jacobi_fp64_mt(ro, ci, iters=30)
    assert it == 30
    assert _max_rel_err(runs[0], ref) <= 1e-5


def test_pr_pull_converges_and_stage_api(gpu):
    G = g.Graph.rmat(12, 8)
    ro, ci = G.row_offsets, G.col_indices
    part = G.partition_edge_balanced(3)
    with g.Context(G, part, num_memory=3) as ctx:
        ctx.set_algo(g.GRD_PR_PULL, max_rounds=100, tolerance=1e-7)
        ctx.init()
        st = ctx.run()
        ref, it, _ = O.pr_jacobi_fp64(ro, ci, iters=100, tol=1e-7)
        assert st["converged"] == 1 and abs(st["rounds"] - it) <= 1  # FP64 may stop one iteration apart
        P = O.PrJacobi(ro, ci, threads=2)  # the same FP32-Kahan arithmetic and stop rule
        P.init()
        assert P.iterate(100, 1e-7)[0] == st["rounds"]
        full = ctx.read_ranks()
        # the same iterations through the per-stage API
        ctx.init()
        r = 0
        while ctx.round() != 0:
            r += 1
        assert r + 1 == st["rounds"]
        np.testing.assert_array_equal(ctx.read_ranks(), full)


def test_reference_cpu_case_pagerank_rmat16(gpu, tmp_path):
    """The reference's own CPU-runnable case: plain PageRank (delta push,
    damping 0.85) for 20 iterations on seeded RMAT-16 ef16, written as
    .mtx, 1 compute + 1 memory partition.  Through the .mtx reader, the
    plugin driver and the C ABI against the oracle."""
    import subprocess
    from pathlib import Path
    G0 = g.Graph.rmat(16, 16, seed=g.rmat_seed(16, 16))
    path = tmp_path / "rmat16.mtx"
    G0.write_mtx(str(path))
    G = g.Graph.read_mtx(str(path))
    np.testing.assert_array_equal(G.row_offsets, G0.row_offsets)
    np.testing.assert_array_equal(G.col_indices, G0.col_indices)
    ref = O.run(O.ORC_PR_DELTA, G.row_offsets, G.col_indices, max_rounds=20)
    assert ref["stats"]["rounds"] == 20
    with g.Context(G, None, num_memory=1) as ctx:
        ctx.set_algo(g.GRD_PR_DELTA, max_rounds=20)
        ctx.init()
        st = ctx.run()
        assert st["rounds"] == 20
        np.testing.assert_allclose(ctx.read_ranks(), ref["ranks"], rtol=1e-4, atol=2e-5)
    cli = Path(g.__file__).resolve().parent / "_build" / "grudon"
    if cli.exists():
        r = subprocess.run([str(cli), "-g", str(path), "-c", "1", "-m", "1", "-a", "pr", "--max-rounds", "20"],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        assert "STAT PageRank Iterations 20" in r.stdout, r.stdout
        total = float(next(l for l in r.stdout.splitlines() if l.startswith("CHECKSUM")).split()[1])
        assert abs(total - float(ref["ranks"].astype(np.float64).sum())) < 1e-3 * max(1.0, total)


@pytest.mark.parametrize("algo,oalgo", [(g.GRD_SSSP_HOP, O.ORC_SSSP_HOP), (g.GRD_SSSP_W, O.ORC_SSSP_W),
                                        (g.GRD_CC, O.ORC_CC)])
@pytest.mark.parametrize("offload", [g.GRD_OFFLOAD_NDP, g.GRD_OFFLOAD_NONE], ids=["ndp", "no-offload"])
def test_small_rounds_run_back_to_back_in_one_kernel(gpu, algo, oalgo, offload):
    """A high-diameter graph: its small rounds run inside one kernel launch of
    the device-driven loop, with the same results and round statistics as
    the host-driven loop (one launch per round) and the oracle."""
    G = g.Graph.grid(96, seed=4)
    part = G.partition_edge_balanced(2)
    ref = O.Layout(G.row_offsets, G.col_indices, G.weights, part, 2).run(
        oalgo, offload=O.ORC_OFFLOAD_NONE if offload == g.GRD_OFFLOAD_NONE else O.ORC_OFFLOAD_NDP)
    with g.Context(G, part, num_memory=2) as ctx:
        for cap in (1000, 37):
            ctx.set_algo(algo, offload=offload, max_rounds=cap)
            ctx.init()
            hs = ctx.run(host_loop=True)
            hp = ctx.read_props()
            ctx.init()
            ds = ctx.run()
            np.testing.assert_array_equal(ctx.read_props(), hp)
            for k in ("rounds", "converged", "edges_scanned", "bytes_synced", "reference_bytes_moved",
                      "push_rounds", "pull_rounds", "actives_total", "push_actives", "no_offload_rounds"):
                assert ds[k] == hs[k], k
            if cap == 1000:
                np.testing.assert_array_equal(hp, ref["props"])
                assert ds["rounds"] == ref["stats"]["rounds"] > 100
                if algo != g.GRD_CC:  # SSSP's wavefront stays small: far fewer than three launches a round
                    assert ds["kernel_launches"] < 2 * ds["rounds"]
            else:
                assert ds["rounds"] == 37 and ds["converged"] == 0


def test_cc_sssp_rmat20_with_hub_rows_bit_exact(gpu):
    """RMAT-20, 1C+3M: rows above the hub threshold exist (so the hub kernel
    runs) and CC labels / weighted SSSP distances, round counts and the
    verify() invariants equal the oracle's restated round protocol."""
    import os
    threads = os.cpu_count() or 1
    for algo, oalgo, sym in ((g.GRD_CC, O.ORC_CC, True), (g.GRD_SSSP_W, O.ORC_SSSP_W, False)):
        G = g.Graph.rmat(20, 16, symmetrize=sym, weighted=not sym)
        part = G.partition_edge_balanced(3)
        ref = O.Layout(G.row_offsets, G.col_indices, G.weights, part, 3).run(oalgo, threads=threads)
        with g.Context(G, part, num_memory=3) as ctx:
            assert len(ctx.read_layout("hubs")) > 0
            ctx.set_algo(algo)
            ctx.init()
            st = ctx.run()
            np.testing.assert_array_equal(ctx.read_props(), ref["props"])
            assert st["rounds"] == ref["stats"]["rounds"]
            assert st["bytes_synced"] == ref["stats"]["bytes_synced"]
            assert ctx.verify()["errors"] == 0


def test_pr_pull_reproducible_and_tight(gpu):
    """PR_PULL sums every list in a fixed order and reduces the residual in a
    fixed order: two runs give the same ranks, residual and iteration count
    bit for bit, within 1e-5 relative error of FP64 Jacobi and one FP32 ulp
    scale of the host FP32-Kahan restatement."""
    G = g.Graph.rmat(16, 16)
    ro, ci = G.row_offsets, G.col_indices
    part = G.partition_edge_balanced(3)
    with g.Context(G, part, num_memory=3) as ctx:
        ctx.set_algo(g.GRD_PR_PULL, max_rounds=100, tolerance=1e-7)
        runs = []
        for _ in range(2):
            ctx.init()
            st = ctx.run()
            runs.append((st["rounds"], st["last_residual"], ctx.read_ranks()))
        assert runs[0][0] == runs[1][0] and runs[0][1] == runs[1][1]
        np.testing.assert_array_equal(runs[0][2], runs[1][2])
        it = runs[0][0]
        ref, _, _ = O.pr_jacobi_fp64(ro, ci, iters=it)
        assert _max_rel_err(runs[0][2], ref) <= 1e-5
        P = O.PrJacobi(ro, ci, threads=2)
        P.init()
        assert P.iterate(100, 1e-7)[0] == it
        assert _max_rel_err(runs[0][2], P.ranks().astype(np.float64)) <= 1e-5
