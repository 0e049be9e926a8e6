"""Batched right-hand sides and the SpMV adjoint through the C ABI.

Forward Y = A X and backward dX = A^T G, dA[e] = <G[row(e)], X[col(e)]> against scipy in FP64:
|err| <= 1e-5 x (the matching sum of |terms|), bit-reproducible across runs, gradcheck of the thin
autograd wrapper, and a random-direction central difference of L = <A X, R> in FP64."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _matrix(g, vals):
    import scipy.sparse as sp

    # Copies: scipy may canonicalise (sum duplicate arcs) in place on the arrays it is given.
    return sp.csr_matrix((vals.astype(np.float64), g.col.copy(), g.offsets.copy()), shape=(g.V, g.V))


def _hubby():
    rng = np.random.default_rng(4)
    V = 3000
    src = [5] * 2000 + [6] * 600 + [7] * 513 + list(rng.integers(0, V, 20000))
    dst = list(rng.integers(0, V, 2000 + 600 + 513 + 20000))
    return dpg.csr_from_arcs(V, src, dst)


@pytest.fixture(scope="module")
def cases():
    return {"rmat12": dpg.rmat_csr(12, 16, seed=12, weights=False), "hubby": _hubby()}


@pytest.mark.parametrize("name", ["rmat12", "hubby"])
@pytest.mark.parametrize("nrhs", [1, 7, 32, 64, 100])
def test_spmm_and_backward_vs_fp64(ctx, cases, name, nrhs):
    import torch

    g = cases[name]
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(nrhs)
    vals = np.exp(rng.normal(0, 1, g.E)).astype(np.float32)
    X = rng.uniform(-1, 1, (g.V, nrhs)).astype(np.float32)
    G = rng.uniform(-1, 1, (g.V, nrhs)).astype(np.float32)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    tv, tX, tG = (torch.from_numpy(a).to(dev) for a in (vals, X, G))
    Y = torch.empty((g.V, nrhs), device=dev)
    dX = torch.empty((g.V, nrhs), device=dev)
    dA = torch.empty(g.E, device=dev)
    dpg.spmm_dev(ctx, dg, tv.data_ptr(), nrhs, tX.data_ptr(), Y.data_ptr())
    dpg.spmv_bwd_dev(ctx, dg, tv.data_ptr(), nrhs, tX.data_ptr(), tG.data_ptr(), dX.data_ptr(), dA.data_ptr())
    ctx.synchronize()
    A = _matrix(g, vals)
    Aabs = abs(A)
    X64, G64 = X.astype(np.float64), G.astype(np.float64)
    assert np.all(np.abs(Y.cpu().numpy() - A @ X64) <= TOL * (Aabs @ np.abs(X64)) + 1e-30)
    assert np.all(np.abs(dX.cpu().numpy() - A.T @ G64) <= TOL * (Aabs.T @ np.abs(G64)) + 1e-30)
    rows = np.repeat(np.arange(g.V), np.diff(g.offsets))
    dA64 = np.sum(G64[rows] * X64[g.col], axis=1)
    mag = np.sum(np.abs(G64[rows] * X64[g.col]), axis=1)
    assert np.all(np.abs(dA.cpu().numpy() - dA64) <= TOL * mag + 1e-30)


def test_backward_is_bit_reproducible(ctx, cases):
    import torch

    g = cases["hubby"]
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(0)
    tv = torch.from_numpy(rng.uniform(0, 1, g.E).astype(np.float32)).to(dev)
    tX = torch.from_numpy(rng.uniform(-1, 1, (g.V, 64)).astype(np.float32)).to(dev)
    tG = torch.from_numpy(rng.uniform(-1, 1, (g.V, 64)).astype(np.float32)).to(dev)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    outs = []
    for _ in range(2):
        dX = torch.empty((g.V, 64), device=dev)
        dA = torch.empty(g.E, device=dev)
        dpg.spmv_bwd_dev(ctx, dg, tv.data_ptr(), 64, tX.data_ptr(), tG.data_ptr(), dX.data_ptr(), dA.data_ptr())
        ctx.synchronize()
        outs.append((dX.cpu().numpy().view(np.uint32), dA.cpu().numpy().view(np.uint32)))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_gradcheck_small_graph(ctx):
    import torch

    from smdp_gb300.autograd import spmm

    g = dpg.rmat_csr(5, 4, seed=3, weights=False)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(1)
    vals = torch.tensor(rng.uniform(0.5, 1.5, g.E), dtype=torch.float32, device=dev, requires_grad=True)
    X = torch.tensor(rng.uniform(-1, 1, (g.V, 3)), dtype=torch.float32, device=dev, requires_grad=True)
    fn = lambda v, x: spmm(ctx, dg, v, x)  # noqa: E731
    assert torch.autograd.gradcheck(fn, (vals, X), eps=1e-2, atol=2e-3, rtol=2e-2, nondet_tol=0.0)


def test_random_direction_central_difference_fp64(ctx):
    import torch

    from smdp_gb300.autograd import spmm

    g = dpg.rmat_csr(14, 16, seed=14, weights=False)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(2)
    vals_np = np.exp(rng.normal(0, 1, g.E)).astype(np.float32)
    X_np = rng.uniform(-1, 1, (g.V, 64)).astype(np.float32)
    R_np = rng.uniform(-1, 1, (g.V, 64)).astype(np.float32)
    vals = torch.tensor(vals_np, device=dev, requires_grad=True)
    X = torch.tensor(X_np, device=dev, requires_grad=True)
    Y = spmm(ctx, dg, vals, X)
    (Y * torch.from_numpy(R_np).to(dev)).sum().backward()
    dv = rng.normal(0, 1, g.E)
    dXd = rng.normal(0, 1, (g.V, 64))
    ana = float(np.dot(vals.grad.cpu().numpy().astype(np.float64), dv) +
                np.sum(X.grad.cpu().numpy().astype(np.float64) * dXd))
    import scipy.sparse as sp

    def loss(vv, xx):
        A = sp.csr_matrix((vv, g.col.copy(), g.offsets.copy()), shape=(g.V, g.V))
        return float(np.sum((A @ xx) * R_np.astype(np.float64)))

    eps = 1e-3
    v64, x64 = vals_np.astype(np.float64), X_np.astype(np.float64)
    num = (loss(v64 + eps * dv, x64 + eps * dXd) - loss(v64 - eps * dv, x64 - eps * dXd)) / (2 * eps)
    assert abs(ana - num) <= 1e-4 * max(1.0, abs(num))


def test_backward_full_size_rmat22_64rhs_vs_fp64_sample(ctx):
    """The stated adjoint configuration at its size: R-MAT scale 22 (67,108,864 arcs), FP32 values
    lognormal(0, 1), 64 right-hand sides. dX = A^T G and dA are checked in FP64 on a seeded 1 % of
    the vertices (every arc into each sampled vertex) and 1 % of the arcs, each entry within
    1e-5 x its sum of |terms|."""
    import torch

    g = dpg.rmat_csr(22, 16, seed=22, weights=False)
    V, E, nrhs = g.V, g.E, 64
    dev = torch.device("cuda", 0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)
    vals = torch.exp(torch.randn(E, device=dev, generator=gen))
    X = torch.rand((V, nrhs), device=dev, generator=gen) * 2 - 1
    G = torch.rand((V, nrhs), device=dev, generator=gen) * 2 - 1
    dX = torch.empty((V, nrhs), device=dev)
    dA = torch.empty(E, device=dev)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    dpg.spmv_bwd_dev(ctx, dg, vals.data_ptr(), nrhs, X.data_ptr(), G.data_ptr(), dX.data_ptr(), dA.data_ptr())
    ctx.synchronize()
    rng = np.random.default_rng(22)
    v_np = vals.cpu().numpy().astype(np.float64)
    # dX rows of a 1 % vertex sample, from the transposed CSR (arc permutation gives each in-arc's value).
    t_off, t_col, t_arc = dpg.csr_transpose_perm(V, g.offsets, g.col)
    js = np.sort(rng.choice(V, V // 100, replace=False))
    lo, hi = t_off[js].astype(np.int64), t_off[js + 1].astype(np.int64)
    cnt = hi - lo
    idx = np.repeat(lo - np.cumsum(cnt) + cnt, cnt) + np.arange(cnt.sum())
    seg = np.repeat(np.arange(js.size), cnt)
    G_rows = G[torch.from_numpy(t_col[idx].astype(np.int64)).to(dev)].cpu().numpy().astype(np.float64)
    terms = v_np[t_arc[idx]][:, None] * G_rows
    exp = np.zeros((js.size, nrhs))
    mag = np.zeros((js.size, nrhs))
    np.add.at(exp, seg, terms)
    np.add.at(mag, seg, np.abs(terms))
    got = dX[torch.from_numpy(js.astype(np.int64)).to(dev)].cpu().numpy()
    assert np.all(np.abs(got - exp) <= TOL * mag + 1e-30)
    # dA on a 1 % arc sample.
    es = np.sort(rng.choice(E, E // 100, replace=False))
    rows = np.searchsorted(g.offsets, es, side="right") - 1
    Gr = G[torch.from_numpy(rows.astype(np.int64)).to(dev)].cpu().numpy().astype(np.float64)
    Xc = X[torch.from_numpy(g.col[es].astype(np.int64)).to(dev)].cpu().numpy().astype(np.float64)
    prod = Gr * Xc
    got_a = dA[torch.from_numpy(es.astype(np.int64)).to(dev)].cpu().numpy()
    assert np.all(np.abs(got_a - prod.sum(axis=1)) <= TOL * np.abs(prod).sum(axis=1) + 1e-30)


def test_group_and_general_paths_agree(ctx, cases):
    """nrhs = 64 with 16-byte aligned rows takes the group kernels (float4 rows, one pass for dX and
    dA); the same data at a 4-byte offset takes the general kernels. Both within the FP64 bound, and
    the Inf rows of a vertex that no arc touches stay out of every result."""
    import torch

    h = cases["hubby"]
    # The hub graph plus one isolated vertex, whose rows of X and G hold Inf.
    g = dpg.csr_from_arcs(h.V + 1, np.repeat(np.arange(h.V), np.diff(h.offsets)), h.col)
    lonely = h.V
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(9)
    nrhs = 64
    vals = np.exp(rng.normal(0, 1, g.E)).astype(np.float32)
    X = rng.uniform(-1, 1, (g.V, nrhs)).astype(np.float32)
    G = rng.uniform(-1, 1, (g.V, nrhs)).astype(np.float32)
    X[lonely] = np.inf
    G[lonely] = np.inf
    dg = dpg.Graph(ctx, g.offsets, g.col)
    tv = torch.from_numpy(vals).to(dev)
    outs = {}
    for off in (0, 1):
        bX = torch.zeros(g.V * nrhs + off, device=dev)
        bG = torch.zeros(g.V * nrhs + off, device=dev)
        bX[off:] = torch.from_numpy(X.ravel()).to(dev)
        bG[off:] = torch.from_numpy(G.ravel()).to(dev)
        dX = torch.empty(g.V * nrhs + off, device=dev)
        dA = torch.empty(g.E, device=dev)
        Y = torch.empty(g.V * nrhs + off, device=dev)
        dpg.spmv_bwd_dev(ctx, dg, tv.data_ptr(), nrhs, bX[off:].data_ptr(), bG[off:].data_ptr(), dX[off:].data_ptr(),
                         dA.data_ptr())
        dpg.spmm_dev(ctx, dg, tv.data_ptr(), nrhs, bX[off:].data_ptr(), Y[off:].data_ptr())
        ctx.synchronize()
        outs[off] = (dX[off:].view(g.V, nrhs).cpu().numpy(), dA.cpu().numpy(), Y[off:].view(g.V, nrhs).cpu().numpy())
    A = _matrix(g, vals)
    Aabs = abs(A)
    X64 = np.where(np.isinf(X), 0, X).astype(np.float64)
    G64 = np.where(np.isinf(G), 0, G).astype(np.float64)
    rows = np.repeat(np.arange(g.V), np.diff(g.offsets))
    keep = np.ones(g.V, bool)
    keep[lonely] = False
    for off, (dX, dA, Y) in outs.items():
        assert np.all(np.abs(dX - A.T @ G64)[keep] <= TOL * (Aabs.T @ np.abs(G64))[keep] + 1e-30), off
        assert np.all(np.abs(Y - A @ X64)[keep] <= TOL * (Aabs @ np.abs(X64))[keep] + 1e-30), off
        prod = G64[rows] * X64[g.col]
        assert np.all(np.abs(dA - prod.sum(axis=1)) <= TOL * np.abs(prod).sum(axis=1) + 1e-30), off
        assert np.all(np.isfinite(dA))
