"""Host graph tools and the layout contract (CPU only)."""
import numpy as np
import pytest

import grudon_gb300 as g
from oracle import ffi as O


def _edges(G):
    src = np.repeat(np.arange(G.num_vertices, dtype=np.int64), np.diff(G.row_offsets.astype(np.int64)))
    return src, G.col_indices.astype(np.int64)


def test_rmat_deterministic_and_clean():
    a = g.Graph.rmat(12, 16, weighted=True, threads=1)
    b = g.Graph.rmat(12, 16, weighted=True, threads=7)
    np.testing.assert_array_equal(a.row_offsets, b.row_offsets)
    np.testing.assert_array_equal(a.col_indices, b.col_indices)
    np.testing.assert_array_equal(a.weights, b.weights)
    s, d = _edges(a)
    assert np.all(s != d)
    key = s * a.num_vertices + d
    assert np.all(np.diff(key) > 0)  # sorted rows, no duplicates
    assert a.weights.min() >= 1 and a.weights.max() <= 255
    assert a.seed == g.rmat_seed(12, 16)
    # vertex 0 is the hub (no relabelling)
    assert np.argmax(np.diff(a.row_offsets.astype(np.int64))) == 0


def test_symmetrize_and_er_grid():
    S = g.Graph.rmat(10, 8, symmetrize=True)
    s, d = _edges(S)
    fwd = set(zip(s.tolist(), d.tolist()))
    assert all((y, x) in fwd for x, y in fwd)
    E = g.Graph.er(3000, 4, seed=3)
    assert 0 < E.num_edges <= 12000
    K = g.Graph.grid(5)
    assert K.num_vertices == 25 and K.num_edges == 2 * 2 * 5 * 4


def test_gr_and_mtx_round_trip(tmp_path):
    G = g.Graph.rmat(9, 8, weighted=True)
    for ext, wr, rd in (("gr", G.write_gr, g.Graph.read_gr), ("mtx", G.write_mtx, g.Graph.read_mtx)):
        p = str(tmp_path / f"g.{ext}")
        wr(p)
        H = rd(p)
        np.testing.assert_array_equal(G.row_offsets, H.row_offsets)
        np.testing.assert_array_equal(G.col_indices, H.col_indices)
        np.testing.assert_array_equal(G.weights, H.weights)


def test_corrupt_graph_files_are_rejected(tmp_path):
    p = tmp_path / "bad.gr"
    p.write_bytes(b"\x01\x00\x00")
    with pytest.raises(g.GrdError):
        g.Graph.read_gr(str(p))
    with pytest.raises(g.GrdError):
        g.Graph.read_gr(str(tmp_path / "missing.gr"))
    q = tmp_path / "bad.mtx"
    q.write_text("%%MatrixMarket matrix coordinate pattern general\n3 3 1\n7 1\n")
    with pytest.raises(g.GrdError):
        g.Graph.read_mtx(str(q))


def test_partition_file_round_trip_and_errors(tmp_path):
    G = g.Graph.rmat(10, 8)
    part = G.partition_edge_balanced(3)
    assert set(np.unique(part)) == {0, 1, 2}
    assert np.all(np.diff(part.astype(np.int64)) >= 0)  # contiguous ranges
    edges = np.bincount(part, weights=np.diff(G.row_offsets.astype(np.int64)) + 1)
    assert edges.max() < 2.0 * edges.mean()
    p = str(tmp_path / "parts.txt")
    g.write_partition_file(part, p)
    np.testing.assert_array_equal(g.read_partition_file(p, G.num_vertices, 3), part)
    with pytest.raises(g.GrdError):  # ids out of range for M = 2
        g.read_partition_file(p, G.num_vertices, 2)
    with pytest.raises(g.GrdError):  # short file
        g.read_partition_file(p, G.num_vertices + 5, 3)


@pytest.mark.parametrize("num_memory", [1, 2, 3, 5])
def test_layout_slot_order_matches_oracle(num_memory):
    """Translation-slot order (owned ascending, then proxies ascending),
    src/DistributedGraph.cpp:579-588, 630-758."""
    G = g.Graph.rmat(11, 8)
    part = G.partition_edge_balanced(num_memory) if num_memory > 1 else None
    total_owned = 0
    for p in range(num_memory):
        slots, n_owned = g.layout_preview(G, part, num_memory, p)
        ref, ref_owned = O.layout_slots(G.row_offsets, G.col_indices, part, num_memory, p)
        np.testing.assert_array_equal(slots, ref)
        assert n_owned == ref_owned
        total_owned += n_owned
    assert total_owned == G.num_vertices


def test_layout_rejects_bad_input():
    G = g.Graph.rmat(8, 4)
    with pytest.raises(g.GrdError):
        g.layout_preview(G, np.full(G.num_vertices, 7, dtype=np.uint32), 3, 0)
    with pytest.raises(g.GrdError):
        g.layout_preview(G, None, 0, 0)


@pytest.mark.parametrize("scale,ef,sym,weighted", [(6, 4, False, False), (9, 8, True, True), (12, 16, False, True),
                                                   (13, 16, True, False), (14, 32, False, True)])
def test_oracle_generator_equals_product(scale, ef, sym, weighted):
    """The oracle's restated RMAT generator (its own key sort) gives the
    product generator's CSR, weights and edge-balanced partition bit for bit,
    so the CPU reference arm runs on the benchmark's graphs without the
    product library."""
    from oracle import ffi as O
    seed = g.rmat_seed(scale, ef)
    assert O.rmat_seed(scale, ef) == seed
    G = g.Graph.rmat(scale, ef, seed=seed, symmetrize=sym, weighted=weighted)
    ro, col, w = O.gen_rmat(scale, ef, seed=seed, symmetrize=sym, weighted=weighted)
    np.testing.assert_array_equal(G.row_offsets, ro)
    np.testing.assert_array_equal(G.col_indices, col)
    if weighted:
        np.testing.assert_array_equal(G.weights, w)
    else:
        assert w is None
    np.testing.assert_array_equal(G.partition_edge_balanced(3), O.partition_edge_balanced(ro, 3))
    assert O.csr_checksum(G.row_offsets, G.col_indices, G.weights) == O.csr_checksum(ro, col, w)
