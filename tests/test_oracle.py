"""The oracle (CPU restatement of the reference protocol) pinned against the
golden fixtures, independent textbook oracles and the reference's verify()
invariants.  CPU only."""
import json
from pathlib import Path

import numpy as np
import pytest

import grudon_gb300 as g
from oracle import ffi as O

GOLDEN = json.loads((Path(__file__).parent / "golden" / "tiny_graphs.json").read_text())


@pytest.mark.parametrize("fx", GOLDEN, ids=[f["name"] for f in GOLDEN])
def test_golden_fixtures(fx):
    ro, ci, w = fx["row_offsets"], fx["col_indices"], fx["weights"]
    assert list(O.run(O.ORC_CC, ro, ci)["props"]) == fx["cc"]
    hop = O.run(O.ORC_SSSP_HOP, ro, ci)
    assert list(hop["props"]) == fx["hop"]
    assert list(O.run(O.ORC_SSSP_W, ro, ci, w)["props"]) == fx["sssp_w"]
    if "hop_rounds" in fx:
        assert hop["stats"]["rounds"] == fx["hop_rounds"]
    if "pr" in fx:
        r = O.run(O.ORC_PR_DELTA, ro, ci)
        np.testing.assert_allclose(r["ranks"], fx["pr"], atol=1e-6)
        assert r["stats"]["rounds"] == fx["pr_rounds"]


@pytest.mark.parametrize("num_memory", [1, 2, 3])
@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_vs_textbook(num_memory, seed):
    G = g.Graph.er(1500, 3, seed=seed, symmetrize=True, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    kw = dict(mirror=part, num_memory=num_memory)
    np.testing.assert_array_equal(O.run(O.ORC_CC, ro, ci, **kw)["props"], O.cc_union_find(ro, ci))
    np.testing.assert_array_equal(O.run(O.ORC_SSSP_HOP, ro, ci, **kw)["props"], O.bfs(ro, ci, 0))
    np.testing.assert_array_equal(O.run(O.ORC_SSSP_W, ro, ci, w, **kw)["props"], O.dijkstra(ro, ci, w, 0))


def test_oracle_pagerank_fixed_point():
    G = g.Graph.rmat(11, 8)
    ro, ci = G.row_offsets, G.col_indices
    r = O.run(O.ORC_PR_DELTA, ro, ci)
    fp, _, _ = O.pr_jacobi_fp64(ro, ci, iters=400)
    # delta push leaves at most TOL-sized residues per vertex
    assert np.max(np.abs(r["ranks"] - fp)) < 5e-4
    fp2, _, _ = O.pr_jacobi_fp64_mt(ro, ci, iters=400, threads=3)
    np.testing.assert_array_equal(fp, fp2)


def test_threaded_oracle_matches_sequential_for_min_algorithms():
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    part = G.partition_edge_balanced(3)
    for a in (O.ORC_CC, O.ORC_SSSP_HOP, O.ORC_SSSP_W):
        s = O.run(a, ro, ci, w, mirror=part, num_memory=3, threads=1)
        t = O.run(a, ro, ci, w, mirror=part, num_memory=3, threads=4)
        np.testing.assert_array_equal(s["props"], t["props"])
        assert s["stats"] == t["stats"]


def test_reference_verify_invariants():
    """cc.cpp:139-177 (equal labels across every edge) and sssp.cpp:145-189
    (dist[dst] <= dist[src] + 1) on a directed graph."""
    G = g.Graph.rmat(11, 8, symmetrize=True)
    ro, ci = G.row_offsets.astype(np.int64), G.col_indices
    lab = O.run(O.ORC_CC, ro, ci)["props"]
    src = np.repeat(np.arange(G.num_vertices), np.diff(ro))
    assert np.all(lab[src] == lab[ci])
    D = g.Graph.rmat(11, 8)
    ro, ci = D.row_offsets.astype(np.int64), D.col_indices
    d = O.run(O.ORC_SSSP_HOP, ro, ci)["props"].astype(np.int64)
    src = np.repeat(np.arange(D.num_vertices), np.diff(ro))
    reach = d[src] != 0xFFFFFFFF
    assert np.all(d[ci][reach] <= d[src][reach] + 1)


def test_byte_accounting_formula():
    """TotalBytesMoved of the reference counts the bitvector as size_bytes()
    elements of MPI_UINT64_T (x8, src/GraphAlgorithm.cpp:251-265)."""
    fx = GOLDEN[0]
    r = O.run(O.ORC_CC, fx["row_offsets"], fx["col_indices"])
    st = r["stats"]
    # n=4 -> one 64-bit word per direction per round
    rounds = st["rounds"]
    words = 2 * rounds * 8
    values = st["bytes_synced"] - words
    assert st["reference_bytes_moved"] == 8 * words + values
