"""Degenerate inputs through the newer entry points: graphs without arcs, single vertices, a batch
holding arcless graphs, and the device transpose of an empty arc set. Every call either succeeds
with the mathematically expected result or returns an error; none may fault."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu


def _arcless(V):
    z = np.zeros(0, np.int32)
    return dpg.csr_from_arcs(V, z, z, z)


def test_transpose_without_arcs(ctx):
    import torch

    g = _arcless(5)
    off = torch.from_numpy(g.offsets).cuda()
    col = torch.zeros(1, dtype=torch.int32, device="cuda")
    t_off = torch.full((6,), -1, dtype=torch.int32, device="cuda")
    t_col = torch.zeros(1, dtype=torch.int32, device="cuda")
    dpg.csr_transpose_dev(ctx, 5, 0, off.data_ptr(), col.data_ptr(), t_off.data_ptr(), t_col.data_ptr())
    ctx.synchronize()
    assert t_off.cpu().tolist() == [0] * 6


def test_adjoint_and_spmm_without_arcs(ctx):
    import torch

    g = _arcless(4)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    X = torch.rand((4, 3), device="cuda")
    G = torch.rand((4, 3), device="cuda")
    Y = torch.full((4, 3), 7.0, device="cuda")
    dX = torch.full((4, 3), 7.0, device="cuda")
    vals = torch.zeros(1, device="cuda")
    dpg.spmm_dev(ctx, dg, vals.data_ptr(), 3, X.data_ptr(), Y.data_ptr())
    dpg.spmv_bwd_dev(ctx, dg, vals.data_ptr(), 3, X.data_ptr(), G.data_ptr(), dX.data_ptr(), None)
    ctx.synchronize()
    assert not Y.any() and not dX.any()


def test_weighted_pagerank_all_dangling(ctx):
    import torch

    g = _arcless(8)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    w = torch.zeros(1, device="cuda")
    seed = torch.ones(8, device="cuda")
    r = torch.empty(8, device="cuda")
    gr = torch.empty(1, device="cuda")
    dpg.pagerank_grad_dev(ctx, dg, w.data_ptr(), seed.data_ptr(), r.data_ptr(), gr.data_ptr(), iterations=50,
                          epsilon=1e-7, adjoint_epsilon=1e-7)
    ctx.synchronize()
    assert np.allclose(r.cpu().numpy(), 1.0 / 8, rtol=1e-6)


def test_batch_with_arcless_and_single_vertex_graphs(ctx):
    import torch

    gs = [_arcless(3), _arcless(1), dpg.rmat_csr(6, 4, seed=6), _arcless(2)]
    b = dpg.Batch(ctx, gs)
    src = np.zeros((len(gs), 2), np.int32)
    src[2] = [1, 2]
    dist = torch.empty(2 * b.V, dtype=torch.int32, device="cuda")
    rank = torch.empty(b.V, dtype=torch.float32, device="cuda")
    b.run(src, dist.data_ptr(), rank.data_ptr(), pr_opts_={"iterations": 5})
    ctx.synchronize()
    d = dist.cpu().numpy().reshape(b.V, 2)
    r = rank.cpu().numpy()
    for k, g in enumerate(gs):
        v0, v1 = int(b.vstart[k]), int(b.vstart[k + 1])
        dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
        for c in range(2):
            assert np.array_equal(d[v0:v1, c], dpg.sssp(ctx, dg, int(src[k, c])))
        assert abs(r[v0:v1].astype(np.float64).sum() - 1.0) < 1e-5


def test_cdp_on_a_vertex_without_arcs(ctx):
    import torch

    g = dpg.csr_from_arcs(3, [1], [2])
    dg = dpg.Graph(ctx, g.offsets, g.col)
    lv = torch.empty(3, dtype=torch.int32, device="cuda")
    for variant in (dpg.CDP_NAIVE, dpg.CDP_WARP, dpg.CDP_BLOCK, dpg.CDP_GRID):
        dpg.bfs_cdp_dev(ctx, dg, 0, variant, lv.data_ptr())
        assert lv.cpu().tolist() == [0, dpg.UNDEFINED_LEVEL, dpg.UNDEFINED_LEVEL]
