"""GPU: golden fixtures through the C ABI, and the C++ GraphAlgorithm plugin
API through the flag-compatible CLI (src/main.cpp flags)."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

import grudon_gb300 as g
from oracle import ffi as O

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = json.loads((ROOT / "tests" / "golden" / "tiny_graphs.json").read_text())
CLI = ROOT / "grudon_gb300" / "_build" / "grudon"


@pytest.mark.parametrize("fx", GOLDEN, ids=[f["name"] for f in GOLDEN])
def test_golden_on_gpu(gpu, fx):
    G = g.Graph.from_csr(fx["row_offsets"], fx["col_indices"], fx["weights"])
    with g.Context(G) as ctx:
        for algo, key in ((g.GRD_CC, "cc"), (g.GRD_SSSP_HOP, "hop"), (g.GRD_SSSP_W, "sssp_w")):
            ctx.set_algo(algo)
            ctx.init()
            st = ctx.run()
            assert list(ctx.read_props()) == fx[key], key
            if key == "hop" and "hop_rounds" in fx:
                assert st["rounds"] == fx["hop_rounds"]
        if "pr" in fx:
            ctx.set_algo(g.GRD_PR_DELTA)
            ctx.init()
            st = ctx.run()
            np.testing.assert_allclose(ctx.read_ranks(), fx["pr"], atol=1e-6)
            assert st["rounds"] == fx["pr_rounds"]


def test_aggregate_values(gpu):
    G = g.Graph.from_edges(4, [0, 1], [1, 2])
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        gids = np.array([3, 3, 2], dtype=np.uint32)
        vals = np.array([1, 0, 5], dtype=np.uint32)
        rc = ctx._lib.grd_aggregate_values(ctx._ctx, gids.ctypes.data_as(g._ffi.u32p),
                                           vals.ctypes.data_as(g._ffi.u32p), 3)
        assert rc == 0
        assert list(ctx.read_updates()) == [0xFFFFFFFF, 0xFFFFFFFF, 5, 0]
        bad = np.array([9], dtype=np.uint32)
        rc = ctx._lib.grd_aggregate_values(ctx._ctx, bad.ctypes.data_as(g._ffi.u32p),
                                           vals.ctypes.data_as(g._ffi.u32p), 1)
        assert rc == g._ffi.GRD_E_INVALID


@pytest.mark.parametrize("schedule", [[], ["--policy", "learned", "--policy-model", "MODEL"],
                                      ["--frontier", "list", "--direction", "push"]], ids=["stages", "learned", "list"])
@pytest.mark.parametrize("algo", ["cc", "sssp", "sssp_w", "pr"])
def test_cli_plugin_api_matches_oracle(gpu, tmp_path, algo, schedule):
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    path = str(tmp_path / "g.gr")
    G.write_gr(path)
    part = G.partition_edge_balanced(3)
    pf = str(tmp_path / "parts.txt")
    g.write_partition_file(part, pf)
    from grudon_gb300 import policy as P
    schedule = [str(P.MODEL_FILE) if a == "MODEL" else a for a in schedule]
    r = subprocess.run([str(CLI), "-g", path, "-c", "1", "-m", "3", "-p", pf, "-a", algo, "--verify"] + schedule,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.splitlines() if line.startswith(("CHECKSUM", "VERIFY")))
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    oalgo = {"cc": O.ORC_CC, "sssp": O.ORC_SSSP_HOP, "sssp_w": O.ORC_SSSP_W, "pr": O.ORC_PR_DELTA}[algo]
    ref = O.run(oalgo, ro, ci, w, mirror=part, num_memory=3)
    iters = int([ln for ln in r.stdout.splitlines() if "Iterations" in ln][0].split()[-1])
    if algo == "pr":
        assert abs(float(out["CHECKSUM"]) - float(ref["ranks"].astype(np.float64).sum())) < 1e-2
        assert abs(iters - ref["stats"]["rounds"]) <= 2
    else:
        p = ref["props"].astype(np.uint64)
        expect = int(p[p != 0xFFFFFFFF].sum())
        assert int(out["CHECKSUM"]) == expect
        assert int(out["VERIFY_ERRORS"]) == 0
        assert iters == ref["stats"]["rounds"]
        moved = int([ln for ln in r.stdout.splitlines() if "TotalBytesMoved" in ln][0].split()[-1])
        assert moved == ref["stats"]["reference_bytes_moved"]


def _host_violations(G, labels, kind):
    ro = G.row_offsets.astype(np.int64)
    src = np.repeat(np.arange(G.num_vertices), np.diff(ro))
    dst = G.col_indices.astype(np.int64)
    lu, lv = labels[src].astype(np.uint64), labels[dst].astype(np.uint64)
    if kind == "cc":
        return int(np.count_nonzero(lu != lv))
    w = G.weights.astype(np.uint64) if kind == "sssp_w" else np.ones(len(dst), dtype=np.uint64)
    reach = lu != 0xFFFFFFFF
    return int(np.count_nonzero(reach & (lv > lu + w)))


def test_device_verify(gpu):
    """grd_verify: the reference's verify() invariants on the device, checked
    against host counts, including on deliberately broken labels."""
    from grudon_gb300.batch import Union
    # two disjoint RMAT graphs: the second one's labels are all above 0
    Gs = Union([g.Graph.rmat(11, 8, symmetrize=True, weighted=True)] * 2).graph
    part = Gs.partition_edge_balanced(3)
    with g.Context(Gs, part, 3) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        ctx.run()
        lab = ctx.read_props()
        r = ctx.verify()
        assert r["errors"] == 0 and r["edges_checked"] == Gs.num_edges
        assert r["count"] == len(np.unique(lab))
        # break one label through the aggregate + update stages
        deg = np.diff(Gs.row_offsets.astype(np.int64))
        gid = int(np.flatnonzero((lab != 0) & (deg > 0))[0])
        gids, vals = np.array([gid], dtype=np.uint32), np.array([0], dtype=np.uint32)
        assert ctx._lib.grd_aggregate_values(ctx._ctx, gids.ctypes.data_as(g._ffi.u32p),
                                             vals.ctypes.data_as(g._ffi.u32p), 1) == 0
        ctx.update()
        lab2 = ctx.read_props()
        assert lab2[gid] == 0
        r = ctx.verify()
        assert r["errors"] == _host_violations(Gs, lab2, "cc") > 0
    Gd = g.Graph.rmat(12, 8, weighted=True)
    with g.Context(Gd, Gd.partition_edge_balanced(3), 3) as ctx:
        for algo, kind in ((g.GRD_SSSP_W, "sssp_w"), (g.GRD_SSSP_HOP, "sssp")):
            ctx.set_algo(algo)
            ctx.init()
            ctx.run()
            d = ctx.read_props()
            r = ctx.verify()
            fin = d[d != 0xFFFFFFFF]
            assert r["errors"] == 0 and r["count"] == len(fin) and r["max_value"] == int(fin.max())
            assert r["edges_checked"] == int(np.diff(Gd.row_offsets.astype(np.int64))[d != 0xFFFFFFFF].sum())
        ctx.set_algo(g.GRD_PR_DELTA)
        ctx.init()
        ctx.run()
        ranks = ctx.read_ranks()
        r = ctx.verify()
        order = np.lexsort((np.arange(len(ranks)), -ranks.astype(np.float64)))[:20]
        assert r["top_ids"] == [int(i) for i in order]
        np.testing.assert_array_equal(np.array(r["top_values"], dtype=np.float32), ranks[order])


@pytest.mark.gpu
def test_async_runs_overlap_and_match(gpu):
    """GRD_RUN_ASYNC: two contexts' loops queued back to back give the same
    results and statistics as blocking runs; calls that change the ctx wait
    for a queued run first."""
    G1 = g.Graph.rmat(13, 8, symmetrize=True, weighted=True)
    G2 = g.Graph.rmat(13, 16, weighted=True)
    with g.Context(G1, G1.partition_edge_balanced(3), num_memory=3) as a, \
            g.Context(G2, G2.partition_edge_balanced(3), num_memory=3) as b:
        a.set_algo(g.GRD_CC)
        b.set_algo(g.GRD_SSSP_W)
        ref = []
        for c in (a, b):
            c.init()
            st = c.run()
            ref.append((c.read_props(), st))
        for c in (a, b):
            c.init()
            c.run(wait=False)
        got = [c.wait() for c in (a, b)]
        for c, (props, st), st2 in zip((a, b), ref, got):
            np.testing.assert_array_equal(c.read_props(), props)
            assert st2["device_loop"] == 1
            for k in ("rounds", "converged", "edges_scanned", "bytes_synced", "reference_bytes_moved",
                      "push_rounds", "pull_rounds", "kernel_launches"):
                assert st2[k] == st[k], k
        # a queued run, then init and set_algo without wait(): both wait for it
        a.init()
        a.run(wait=False)
        a.set_algo(g.GRD_SSSP_HOP)
        a.init()
        st = a.run()
        ref = O.run(O.ORC_SSSP_HOP, G1.row_offsets, G1.col_indices, mirror=G1.partition_edge_balanced(3),
                    num_memory=3)
        np.testing.assert_array_equal(a.read_props(), ref["props"])
        assert st["rounds"] == ref["stats"]["rounds"]
        assert a.wait()["rounds"] == st["rounds"]


@pytest.mark.gpu
def test_upload_sends_byte_weights_and_derives_vertex_arrays(gpu):
    """Weights below 256 travel as bytes and are widened on the device;
    out-degrees and owned slots are derived there.  Re-uploads keep every
    result, and a graph with wide weights still uploads them as u32."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    rng = np.random.default_rng(5)
    wide = g.Graph.from_csr(G.row_offsets, G.col_indices, rng.integers(1, 1_000_000, G.num_edges, dtype=np.uint32))
    part = G.partition_edge_balanced(3)
    sizes = []
    for graph in (G, wide):
        ref = O.run(O.ORC_SSSP_W, graph.row_offsets, graph.col_indices, graph.weights, mirror=part, num_memory=3)
        with g.Context(graph, part, num_memory=3) as ctx, \
                g.Context(graph, part, num_memory=3, device_layout=True) as dctx:
            ctx.set_algo(g.GRD_SSSP_W)
            for _ in range(2):
                sizes.append(ctx.upload())
                ctx.init()
                ctx.run()
                np.testing.assert_array_equal(ctx.read_props(), ref["props"])
            for name in ("wgt", "outdeg", "own_slot"):
                np.testing.assert_array_equal(ctx.read_layout(name), dctx.read_layout(name), err_msg=name)
            np.testing.assert_array_equal(ctx.read_layout("outdeg"), np.diff(graph.row_offsets).astype(np.uint32))
    assert sizes[0] == sizes[1] and sizes[2] == sizes[3]
    assert sizes[2] - sizes[0] == 3 * G.num_edges


@pytest.mark.gpu
def test_pagerank_pull_upload_leaves_out_edges_until_needed(gpu):
    """A Jacobi PageRank ctx re-uploads only what it reads (slot map, row
    offsets, the in-edge sources).  The out-edge columns and the weights
    follow before another algorithm or a layout read needs them, and every
    result stays that of a full upload."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    part = G.partition_edge_balanced(3)
    E = G.num_edges
    with g.Context(G, part, num_memory=3) as ctx, g.Context(G, part, num_memory=3) as ref_ctx:
        ref_ctx.set_algo(g.GRD_PR_PULL, max_rounds=30)
        ref_ctx.init()
        ref_ctx.run()
        ranks = ref_ctx.read_ranks()
        ctx.set_algo(g.GRD_PR_PULL, max_rounds=30)  # builds the in-edge view
        ctx.set_algo(g.GRD_CC)
        full = ctx.upload()
        ctx.set_algo(g.GRD_PR_PULL, max_rounds=30)
        slim = ctx.upload()
        assert full - slim == 4 * E + E + 4 * E  # u32 columns, byte weights, in-edge weights
        ctx.init()
        ctx.run()
        np.testing.assert_array_equal(ctx.read_ranks(), ranks)
        for name in ("col", "wgt", "in_wgt"):
            np.testing.assert_array_equal(ctx.read_layout(name), ref_ctx.read_layout(name), err_msg=name)
        assert ctx.upload() == slim
        for algo in (g.GRD_CC, g.GRD_SSSP_W):  # the columns come back before the push runs
            ctx.set_algo(algo)
            ctx.init()
            ctx.run()
            ref = O.run(O.ORC_CC if algo == g.GRD_CC else O.ORC_SSSP_W, G.row_offsets, G.col_indices,
                        G.weights, mirror=part, num_memory=3)
            np.testing.assert_array_equal(ctx.read_props(), ref["props"])


@pytest.mark.gpu
def test_upload_queued_behind_an_async_run(gpu):
    """The end-to-end pipeline's pattern: each step queues a run and the
    read of its result, then the next step's upload on the same ctx before
    waiting.  The upload lands after the run on the ctx stream; every step's
    result equals the oracle's (CC, weighted SSSP) or the first step's
    (Jacobi PageRank, whose slim upload leaves the out-edges stale)."""
    G = g.Graph.rmat(13, 8, symmetrize=True, weighted=True)
    part = G.partition_edge_balanced(3)
    V = G.num_vertices
    refs = {a: O.run(o, G.row_offsets, G.col_indices, G.weights, mirror=part, num_memory=3)["props"]
            for a, o in ((g.GRD_CC, O.ORC_CC), (g.GRD_SSSP_W, O.ORC_SSSP_W))}
    with g.Context(G, part, num_memory=3) as cc, g.Context(G, part, num_memory=3) as ss, \
            g.Context(G, part, num_memory=3) as pr:
        cc.set_algo(g.GRD_CC)
        ss.set_algo(g.GRD_SSSP_W)
        pr.set_algo(g.GRD_PR_PULL, max_rounds=20, tolerance=0.0)
        outs = [np.empty(V, np.uint32), np.empty(V, np.uint32), np.empty(V, np.float32)]
        first_ranks = None
        for _ in range(3):
            for c in (cc, ss, pr):
                c.wait()
                c.init()
                c.run(wait=False)
            cc.read_props(out=outs[0], wait=False)
            ss.read_props(out=outs[1], wait=False)
            pr.read_ranks(out=outs[2], wait=False)
            for c in (cc, ss, pr):
                c.upload()  # the next step's layout, behind this step's run and read
            for c in (cc, ss, pr):
                c.wait()
                c.synchronize()
            np.testing.assert_array_equal(outs[0], refs[g.GRD_CC])
            np.testing.assert_array_equal(outs[1], refs[g.GRD_SSSP_W])
            if first_ranks is None:
                first_ranks = outs[2].copy()
            np.testing.assert_array_equal(outs[2], first_ranks)


@pytest.mark.gpu
def test_read_into_caller_arrays(gpu):
    """read_props / read_updates / read_ranks fill a caller's array (a
    serving loop keeps pinned result buffers) and refuse one of the wrong
    type or size."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    part = G.partition_edge_balanced(3)
    ref = O.run(O.ORC_SSSP_W, G.row_offsets, G.col_indices, G.weights, mirror=part, num_memory=3)
    V = G.num_vertices
    with g.Context(G, part, num_memory=3) as ctx:
        ctx.set_algo(g.GRD_SSSP_W)
        out = np.zeros(V + 5, dtype=np.uint32)  # larger than needed
        for _ in range(2):
            ctx.init()
            ctx.run()
            assert ctx.read_props(out=out) is out
            np.testing.assert_array_equal(out[:V], ref["props"])
            np.testing.assert_array_equal(ctx.read_updates(out=np.empty(V, np.uint32)), ctx.read_updates())
        with pytest.raises(ValueError):
            ctx.read_props(out=np.zeros(V, dtype=np.int64))
        with pytest.raises(ValueError):
            ctx.read_props(out=np.zeros(V - 1, dtype=np.uint32))
        with pytest.raises(ValueError):
            ctx.read_props(out=np.zeros(2 * V, dtype=np.uint32)[::2])
        ranks = np.empty(V, dtype=np.float32)
        assert ctx.read_ranks(out=ranks) is ranks
        # queued: run and read without waiting, then complete the run
        import torch
        pinned = torch.zeros(V, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        ctx.init()
        ctx.run(wait=False)
        assert ctx.read_props(out=pinned, wait=False) is pinned
        ctx.wait()
        np.testing.assert_array_equal(pinned, ref["props"])
        with pytest.raises(ValueError):
            ctx.read_props(wait=False)
