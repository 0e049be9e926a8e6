"""Thin torch.autograd.Functions over the C-ABI adjoints, used only for gradcheck.

    Y = spmm(ctx, graph, vals, X)      # vals [E], X [V, nrhs] FP32 CUDA tensors
    Y.backward(G)  ->  vals.grad = dA  (dA[e] = <G[row(e)], X[col(e)]>),  X.grad = A^T G

    r = weighted_pagerank(ctx, graph, w, **opts)   # graph = out-adjacency, w [E] > 0
    r.backward(s)  ->  w.grad = dL/dw for dL/dr = s (adjoint fixed point on the out-CSR)

The forward and backward run libdpg.so kernels (dpg_spmm_f32_dev, dpg_spmv_bwd_f32_dev,
dpg_pagerank_grad_f32_dev) on the current torch stream; nothing here computes on the CPU.
"""
from __future__ import annotations

import torch

from . import Context, Graph, pagerank_grad_dev, spmm_dev, spmv_bwd_dev


class _SpMM(torch.autograd.Function):
    @staticmethod
    def forward(fctx, ctx: Context, graph: Graph, vals: torch.Tensor, X: torch.Tensor):
        vals = vals.contiguous().float()
        X = X.contiguous().float()
        nrhs = X.shape[1]
        Y = torch.empty((graph.V, nrhs), dtype=torch.float32, device=X.device)
        ctx.set_stream(torch.cuda.current_stream(X.device).cuda_stream)
        spmm_dev(ctx, graph, vals.data_ptr(), nrhs, X.data_ptr(), Y.data_ptr())
        ctx.synchronize()
        fctx.save_for_backward(vals, X)
        fctx.dpg = (ctx, graph)
        return Y

    @staticmethod
    def backward(fctx, G: torch.Tensor):
        vals, X = fctx.saved_tensors
        ctx, graph = fctx.dpg
        G = G.contiguous().float()
        nrhs = X.shape[1]
        dX = torch.empty_like(X) if fctx.needs_input_grad[3] else None
        dA = torch.empty_like(vals) if fctx.needs_input_grad[2] else None
        ctx.set_stream(torch.cuda.current_stream(G.device).cuda_stream)
        spmv_bwd_dev(ctx, graph, vals.data_ptr(), nrhs, X.data_ptr(), G.data_ptr(),
                     dX.data_ptr() if dX is not None else None, dA.data_ptr() if dA is not None else None)
        ctx.synchronize()
        return None, None, dA, dX


def spmm(ctx: Context, graph: Graph, vals: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    return _SpMM.apply(ctx, graph, vals, X)


class _WeightedPageRank(torch.autograd.Function):
    """The forward runs the gradient entry point with a zero seed (its adjoint loop then stops after
    one sweep); the backward runs it again with the incoming seed. Both solves are deterministic,
    so the backward sees the same ranks as the forward."""

    @staticmethod
    def forward(fctx, ctx: Context, graph: Graph, w: torch.Tensor, opts: dict):
        w = w.contiguous().float()
        r = torch.empty(graph.V, dtype=torch.float32, device=w.device)
        seed = torch.zeros(graph.V, dtype=torch.float32, device=w.device)
        grad = torch.empty_like(w)
        ctx.set_stream(torch.cuda.current_stream(w.device).cuda_stream)
        pagerank_grad_dev(ctx, graph, w.data_ptr(), seed.data_ptr(), r.data_ptr(), grad.data_ptr(), **opts)
        ctx.synchronize()
        fctx.save_for_backward(w)
        fctx.dpg = (ctx, graph, opts)
        return r

    @staticmethod
    def backward(fctx, s: torch.Tensor):
        (w,) = fctx.saved_tensors
        ctx, graph, opts = fctx.dpg
        s = s.contiguous().float()
        r = torch.empty(graph.V, dtype=torch.float32, device=w.device)
        grad = torch.empty_like(w)
        ctx.set_stream(torch.cuda.current_stream(w.device).cuda_stream)
        pagerank_grad_dev(ctx, graph, w.data_ptr(), s.data_ptr(), r.data_ptr(), grad.data_ptr(), **opts)
        ctx.synchronize()
        return None, None, grad, None


def weighted_pagerank(ctx: Context, graph: Graph, w: torch.Tensor, **opts) -> torch.Tensor:
    """Ranks of the weighted PageRank on the out-adjacency graph (see dpg_pagerank_grad_f32_dev);
    opts are pagerank_grad_dev's keyword arguments (damping, total_rank, iterations, epsilon,
    adjoint_epsilon)."""
    return _WeightedPageRank.apply(ctx, graph, w, opts)
