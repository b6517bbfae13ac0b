"""grd_aggregate_values_noalloc — the aggregate entry point for callers that
cannot allocate device memory (a process whose device memory is reserved for
its own pool, or a caller that must not take the allocator's
synchronisation) — against grd_aggregate_values.

Collected last on purpose: it exercises the library's fixed staging array,
and a failure here must not hide results of the other tests.  It passes run
alone in a fresh process (the first call performs the per-device set-up) and
after the rest of the suite.
"""
import numpy as np
import pytest

import grudon_gb300 as g
from grudon_gb300 import _ffi

pytestmark = pytest.mark.gpu

MAX = 1 << 18  # GRD_NOALLOC_MAX_VALUES


def _call(ctx, fn, gids, vals):
    gids = np.ascontiguousarray(gids, dtype=np.uint32)
    vals = np.ascontiguousarray(vals, dtype=np.uint32)
    return fn(ctx._ctx, gids.ctypes.data_as(_ffi.u32p), vals.ctypes.data_as(_ffi.u32p), len(gids))


@pytest.mark.parametrize("algo", [g.GRD_CC, g.GRD_SSSP_W, g.GRD_PR_DELTA])
def test_noalloc_matches_allocating_entry_point_twice(gpu, algo):
    G = g.Graph.rmat(14, 8, weighted=True)
    V = G.num_vertices
    rng = np.random.default_rng(7)
    with g.Context(G) as a, g.Context(G) as b:
        for ctx in (a, b):
            ctx.set_algo(algo)
            ctx.init()
        for call in range(2):  # two calls in a row; the array keeps the last contents
            n = 5000 + 3000 * call
            if algo == g.GRD_PR_DELTA:
                gids = rng.permutation(V)[:n]  # distinct gids: float adds then commute exactly
                vals = rng.random(n, dtype=np.float32).view(np.uint32)
            else:
                gids = rng.integers(0, V, n)  # repeated gids exercise the atomic min
                vals = rng.integers(0, 1 << 30, n)
            assert _call(a, a._lib.grd_aggregate_values, gids, vals) == 0
            assert _call(b, b._lib.grd_aggregate_values_noalloc, gids, vals) == 0
            ua, ub = a.read_updates(), b.read_updates()
            if algo == g.GRD_PR_DELTA:
                np.testing.assert_allclose(ub, ua, rtol=1e-6, atol=0)
            else:
                np.testing.assert_array_equal(ub, ua)
            # the dirty set it leaves behind drives the same update
            fa, fb = a.update(), b.update()
            assert fa == fb
            np.testing.assert_array_equal(a.read_frontier(), b.read_frontier())


def test_noalloc_rejects_oversize_and_bad_ids(gpu):
    G = g.Graph.rmat(10, 4)
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        big = np.zeros(MAX + 1, dtype=np.uint32)
        assert _call(ctx, ctx._lib.grd_aggregate_values_noalloc, big, big) == _ffi.GRD_E_INVALID
        assert b"maximum" in ctx._lib.grd_last_error(ctx._ctx)
        assert _call(ctx, ctx._lib.grd_aggregate_values_noalloc, [G.num_vertices], [1]) == _ffi.GRD_E_INVALID
        full = np.arange(MAX, dtype=np.uint32) % G.num_vertices
        assert _call(ctx, ctx._lib.grd_aggregate_values_noalloc, full, full) == 0


def test_noalloc_allocates_nothing_after_set_up(gpu):
    """After the first call (the per-device address look-up), further calls
    leave the device's free memory unchanged."""
    import torch
    G = g.Graph.rmat(12, 8)
    rng = np.random.default_rng(3)
    with g.Context(G) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        gids = rng.integers(0, G.num_vertices, 4096)
        assert _call(ctx, ctx._lib.grd_aggregate_values_noalloc, gids, gids) == 0
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(2):
            assert _call(ctx, ctx._lib.grd_aggregate_values_noalloc, gids, gids) == 0
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0


def test_noalloc_refuses_an_incomplete_layout_like_the_allocating_one(gpu):
    """A re-ingest that fails part-way leaves the layout incomplete: both
    aggregate entry points then refuse the call."""
    G = g.Graph.rmat(11, 8, symmetrize=True)
    part = G.partition_edge_balanced(2)
    with g.Context(G, part, num_memory=2, device_layout=True) as ctx:
        ctx.set_algo(g.GRD_CC)
        ctx.init()
        swapped = (1 - part).astype(np.uint32)  # other owned and proxy counts
        with pytest.raises(g.GrdError):
            ctx.ingest(G, swapped)
        for fn in (ctx._lib.grd_aggregate_values, ctx._lib.grd_aggregate_values_noalloc):
            assert _call(ctx, fn, [1, 2], [0, 0]) == _ffi.GRD_E_INVALID
