"""Partition layout built on the GPU (grd_ctx_create_ex with
GRD_CREATE_DEVICE_LAYOUT) against the host build: every resident array equal,
the in-edge view included, and runs bit-exact to the oracle."""
import numpy as np
import pytest

import grudon_gb300 as g
from oracle import ffi as O

pytestmark = pytest.mark.gpu

ARRAYS = ["slot_gid", "row_off", "col", "wgt", "outdeg", "own_slot", "hubs"]
IN_ARRAYS = ["in_off", "in_src", "in_wgt", "in_hubs", "in_meds"]


def star_plus_rmat():
    """RMAT-14 plus a vertex linked both ways to 9000 others: a push hub of
    several 4096-edge work items and a pulled in-hub."""
    R = g.Graph.rmat(14, 4, symmetrize=True, weighted=True)
    ro, ci, w = R.row_offsets.astype(np.int64), R.col_indices, R.weights
    V = R.num_vertices + 1
    hub = V - 1
    leaves = np.arange(0, 9000, dtype=np.uint32)
    src = np.concatenate([np.repeat(np.arange(R.num_vertices), np.diff(ro)), leaves,
                          np.full(len(leaves), hub)]).astype(np.int64)
    dst = np.concatenate([ci, np.full(len(leaves), hub, dtype=np.uint32), leaves]).astype(np.uint32)
    wt = np.concatenate([w, np.arange(len(leaves)) % 200 + 1, np.arange(len(leaves)) % 100 + 1]).astype(np.uint32)
    order = np.argsort(src, kind="stable")
    src, dst, wt = src[order], dst[order], wt[order]
    ro2 = np.zeros(V + 1, dtype=np.uint64)
    np.add.at(ro2, src + 1, 1)
    return g.Graph.from_csr(np.cumsum(ro2).astype(np.uint64), dst, wt)


def isolated_er():
    """Directed ER with ~1/3 isolated vertices and V not a multiple of 64."""
    G = g.Graph.er(3001, 2, seed=11, weighted=True)
    ro, ci, w = G.row_offsets.astype(np.int64), G.col_indices, G.weights
    keep = (np.arange(G.num_vertices) % 3 != 0)
    deg = np.diff(ro) * keep
    src = np.repeat(np.arange(G.num_vertices), np.diff(ro))
    m = keep[src]
    ro2 = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    return g.Graph.from_csr(ro2, ci[m], w[m])


GRAPHS = {
    "rmat13_dir": lambda: g.Graph.rmat(13, 16, weighted=True),
    "rmat12_sym": lambda: g.Graph.rmat(12, 8, symmetrize=True, weighted=True),
    "grid50": lambda: g.Graph.grid(50, seed=2),
    "er_isolated": isolated_er,
    "star": star_plus_rmat,
    "unweighted": lambda: g.Graph.rmat(11, 8, symmetrize=True),
}


def partitions(G, M, kind):
    if kind == "naive":
        return None
    if kind == "balanced":
        return G.partition_edge_balanced(M)
    rng = np.random.default_rng(M)
    return rng.integers(0, M, size=G.num_vertices).astype(np.uint32)


CASES = [(1, "naive"), (3, "naive"), (3, "balanced"), (5, "random"), (64, "random")]


def assert_same_layout(a, b, names):
    for n in names:
        np.testing.assert_array_equal(a.read_layout(n), b.read_layout(n), err_msg=n)


@pytest.mark.parametrize("M,kind", CASES, ids=[f"{m}-{k}" for m, k in CASES])
@pytest.mark.parametrize("name", list(GRAPHS))
def test_device_layout_equals_host_layout(gpu, name, M, kind):
    G = GRAPHS[name]()
    part = partitions(G, M, kind)
    with g.Context(G, part, num_memory=M) as h, g.Context(G, part, num_memory=M, device_layout=True) as d:
        for p in range(M):
            assert h.layout_info(p) == d.layout_info(p)
            np.testing.assert_array_equal(h.layout_slots(p), d.layout_slots(p))
        assert_same_layout(h, d, ARRAYS)
        # the in-edge view, built when pull first needs it
        for c in (h, d):
            c.set_algo(g.GRD_PR_PULL, max_rounds=3)
        assert_same_layout(h, d, IN_ARRAYS)
        # the oracle's slot order too
        for p in range(M):
            np.testing.assert_array_equal(
                d.layout_slots(p), O.layout_slots(G.row_offsets, G.col_indices, part, M, p)[0])


@pytest.mark.parametrize("name", ["rmat13_dir", "star", "er_isolated"])
def test_device_layout_runs_bit_exact(gpu, name):
    G = GRAPHS[name]()
    part = G.partition_edge_balanced(3)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    with g.Context(G, part, num_memory=3, device_layout=True) as ctx:
        for algo, oalgo in ((g.GRD_CC, O.ORC_CC), (g.GRD_SSSP_HOP, O.ORC_SSSP_HOP), (g.GRD_SSSP_W, O.ORC_SSSP_W)):
            ref = O.run(oalgo, ro, ci, w, mirror=part, num_memory=3)
            for direction in (g.GRD_DIR_AUTO, g.GRD_DIR_PULL):
                ctx.set_algo(algo, direction=direction)
                ctx.init()
                st = ctx.run()
                np.testing.assert_array_equal(ctx.read_props(), ref["props"])
                assert st["rounds"] == ref["stats"]["rounds"]
                assert st["bytes_synced"] == ref["stats"]["bytes_synced"]


def test_device_layout_pagerank_pull_identical(gpu):
    """PR_PULL sums in-lists in their stored order: identical layouts give
    bit-identical ranks."""
    G = g.Graph.rmat(13, 16)
    part = G.partition_edge_balanced(3)
    out = []
    for dev in (False, True):
        with g.Context(G, part, num_memory=3, device_layout=dev) as ctx:
            ctx.set_algo(g.GRD_PR_PULL, max_rounds=30)
            ctx.init()
            ctx.run()
            out.append(ctx.read_ranks())
    np.testing.assert_array_equal(out[0], out[1])


def test_device_layout_ingest(gpu):
    """grd_ingest rebuilds the layout from a new CSR of the same shape: new
    weights give the new distances; a different shape is refused."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    part = G.partition_edge_balanced(2)
    w2 = (G.weights * 7 % 251 + 1).astype(np.uint32)
    G2 = g.Graph.from_csr(G.row_offsets, G.col_indices, w2)
    with g.Context(G, part, num_memory=2, device_layout=True) as ctx:
        ctx.set_algo(g.GRD_SSSP_W)
        for graph, w in ((G, G.weights), (G2, w2), (G, G.weights)):
            nbytes = ctx.ingest(graph, part)
            assert nbytes == 8 * (G.num_vertices + 1) + 8 * G.num_edges + 4 * G.num_vertices
            ctx.init()
            ctx.run()
            ref = O.run(O.ORC_SSSP_W, G.row_offsets, G.col_indices, w, mirror=part, num_memory=2)
            np.testing.assert_array_equal(ctx.read_props(), ref["props"])
        with pytest.raises(g.GrdError):
            ctx.ingest(g.Graph.rmat(12, 4, symmetrize=True, weighted=True), part)
        with pytest.raises(g.GrdError):
            ctx.upload()


def _create_raw(ro, col, w, part, M):
    """grd_ctx_create_ex on raw arrays (Graph.from_csr would reject them
    first); returns (status, error text) and frees any ctx made."""
    import ctypes as C
    from grudon_gb300 import _ffi
    lib = g.lib()
    ro = np.ascontiguousarray(ro, dtype=np.uint64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    w = None if w is None else np.ascontiguousarray(w, dtype=np.uint32)
    csr = _ffi.grd_csr(len(ro) - 1, len(col), ro.ctypes.data_as(_ffi.u64p), col.ctypes.data_as(_ffi.u32p),
                       None if w is None else w.ctypes.data_as(_ffi.u32p))
    mp = None if part is None else np.ascontiguousarray(part, dtype=np.uint32)
    ctx = C.c_void_p()
    rc = lib.grd_ctx_create_ex(C.byref(csr), None if mp is None else mp.ctypes.data_as(_ffi.u32p), 1, M, 0,
                               _ffi.GRD_CREATE_DEVICE_LAYOUT, C.byref(ctx))
    if ctx.value:
        lib.grd_ctx_destroy(ctx)
    return rc, lib.grd_create_error().decode()


def test_device_layout_rejects_bad_input(gpu):
    """Checked on the device (columns, row monotonicity, mirror ids) or on
    the host (sizes); a refused create leaves nothing behind."""
    G = g.Graph.rmat(10, 4, weighted=True)
    ro, ci, w = G.row_offsets, G.col_indices, G.weights
    rc, why = _create_raw(ro, ci, w, None, 65)
    assert rc != 0 and "64" in why
    bad = ci.copy()
    bad[5] = G.num_vertices
    rc, why = _create_raw(ro, bad, w, None, 2)
    assert rc != 0 and "col_indices" in why
    part = np.zeros(G.num_vertices, dtype=np.uint32)
    part[3] = 9
    rc, why = _create_raw(ro, ci, w, part, 2)
    assert rc != 0 and "mirror" in why
    ro2 = ro.copy()
    k = int(np.argmax(np.diff(ro) > 1))  # a row with 2+ edges: end it early, start the next later
    ro2[k + 1] = ro[k + 2] + 1 if k + 2 < len(ro) - 1 else ro[k + 1]
    if ro2[k + 1] > ro2[k + 2]:
        rc, why = _create_raw(ro2, ci, w, None, 2)
        assert rc != 0 and "monotone" in why
    rc, why = _create_raw(ro, ci, w, None, 2)
    assert rc == 0, why


def test_failed_reingest_leaves_ctx_refusing_until_a_good_one(gpu):
    """A CSR of the same size but other partition counts fails part-way
    through grd_ingest; the ctx then refuses to run until a matching graph is
    ingested again."""
    G = g.Graph.rmat(12, 8, symmetrize=True, weighted=True)
    part = G.partition_edge_balanced(3)
    V = G.num_vertices
    other = g.Graph.from_csr(G.row_offsets, (G.col_indices.astype(np.int64) * 7 + 1) % V, G.weights)
    ref = O.run(O.ORC_SSSP_W, G.row_offsets, G.col_indices, G.weights, mirror=part, num_memory=3)
    with g.Context(G, part, num_memory=3, device_layout=True) as ctx:
        ctx.set_algo(g.GRD_SSSP_W)
        try:
            ctx.ingest(other, part)
            mismatched = False
        except g.GrdError:
            mismatched = True
        if mismatched:
            with pytest.raises(g.GrdError):
                ctx.init()
        ctx.ingest(G, part)
        ctx.init()
        ctx.run()
        np.testing.assert_array_equal(ctx.read_props(), ref["props"])


@pytest.mark.parametrize("V,edges,M", [(1, [], 1), (7, [], 2), (5, [(0, 1), (1, 0), (3, 4)], 3),
                                       (70, [(i, (i * 7 + 3) % 70) for i in range(70)], 64)])
def test_device_layout_tiny_graphs(gpu, V, edges, M):
    """No edges, one vertex, more partitions than owned vertices in some."""
    src = [a for a, _ in edges]
    dst = [b for _, b in edges]
    G = g.Graph.from_edges(V, src, dst, [1 + (a * 3 + b) % 9 for a, b in edges])
    with g.Context(G, None, num_memory=M) as h, g.Context(G, None, num_memory=M, device_layout=True) as d:
        for p in range(M):
            assert h.layout_info(p) == d.layout_info(p)
        assert_same_layout(h, d, ARRAYS)
        for c in (h, d):
            c.set_algo(g.GRD_SSSP_W)
            c.init()
            c.run()
        np.testing.assert_array_equal(h.read_props(), d.read_props())
        for c in (h, d):
            c.set_algo(g.GRD_PR_PULL, max_rounds=3)
        assert_same_layout(h, d, IN_ARRAYS)
