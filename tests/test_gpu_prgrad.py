"""Weighted PageRank and its edge-weight gradient through the C ABI (dpg_pagerank_grad_f32_dev).

Against the FP64 oracle (itself pinned to central differences): ranks within 1e-5 relative, the
per-arc gradient within 1e-5 of its magnitude bound d r[u]/W[u] (|lambda[v]| + |q[u]|), directional
derivatives against FP64 central differences of the loss, bit reproducibility, the fixed-sweep mode,
unit weights against the plain PageRank kernel, gradcheck of the autograd wrapper, and at R-MAT
scale 20 the size-independent properties (ranks sum to T; per-row sum of w * dL/dw is zero)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu
TOL = 1e-5
CONV = dict(damping=0.85, total_rank=1.0, iterations=2000, epsilon=3e-7, adjoint_epsilon=3e-7)


def _dangling_graph():
    # R-MAT scale 11 with every 7th vertex's out-arcs removed (dangling) and a few heavy hubs.
    g = dpg.rmat_csr(11, 16, seed=11, weights=False)
    src = np.repeat(np.arange(g.V), np.diff(g.offsets))
    keep = (src % 7) != 3
    return dpg.csr_from_arcs(g.V, src[keep], g.col[keep])


@pytest.fixture(scope="module")
def cases():
    return {"rmat12": dpg.rmat_csr(12, 16, seed=12, weights=False), "dangling": _dangling_graph()}


def _run(ctx, g, w, seed, **opts):
    import torch

    dev = torch.device("cuda", 0)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    wd = torch.from_numpy(np.ascontiguousarray(w, np.float32)).to(dev)
    sd = torch.from_numpy(np.ascontiguousarray(seed, np.float32)).to(dev)
    r = torch.empty(g.V, device=dev)
    gr = torch.empty(max(g.E, 1), device=dev)
    sweeps = dpg.pagerank_grad_dev(ctx, dg, wd.data_ptr(), sd.data_ptr(), r.data_ptr(), gr.data_ptr(), **opts)
    ctx.synchronize()
    return r.cpu().numpy(), gr.cpu().numpy()[:g.E], sweeps


def _subset_seed(V, rng, frac=0.01):
    s = np.zeros(V)
    s[rng.choice(V, max(1, int(frac * V)), replace=False)] = 1.0
    return s


def _check_vs_fp64(g, w, seed, r, gr):
    """Ranks within TOL relative; each arc's derivative within TOL of its magnitude bound
    d r[u]/W[u] (|lambda[v]| + |q[u]|); L1 error of the gradient within TOL."""
    import scipy.sparse as sp

    import oracle

    r64, lam64, g64 = oracle.pagerank_weighted_grad_f64(g.offsets, g.col, w.astype(np.float64), seed)
    rel = np.abs(r - r64) / r64
    assert rel.max() <= TOL, rel.max()
    rows = np.repeat(np.arange(g.V), np.diff(g.offsets.astype(np.int64)))
    W = np.bincount(rows, w.astype(np.float64), minlength=g.V)
    Wn = np.where(W > 0, W, 1.0)
    A = sp.csr_matrix((w.astype(np.float64), g.col.copy(), g.offsets.copy()), shape=(g.V, g.V))
    q = (A @ lam64) / Wn
    bound = 0.85 * r64[rows] / Wn[rows] * (np.abs(lam64[g.col]) + np.abs(q[rows]))
    err = np.abs(gr.astype(np.float64) - g64)
    assert (err <= TOL * bound + 1e-30).all(), float((err / (bound + 1e-30)).max())
    l1 = np.abs(gr - g64).sum() / np.abs(g64).sum()
    assert l1 <= TOL, l1
    return rows, bound


@pytest.mark.parametrize("name", ["rmat12", "dangling"])
def test_rank_and_gradient_vs_fp64(ctx, cases, name):
    g = cases[name]
    rng = np.random.default_rng(7)
    w = np.exp(rng.standard_normal(g.E)).astype(np.float32)
    seed = _subset_seed(g.V, rng)
    r, gr, (nf, na) = _run(ctx, g, w, seed, **CONV)
    assert 10 < nf < 2000 and 10 < na < 2000
    _check_vs_fp64(g, w, seed, r, gr)


def test_directional_derivative_vs_fp64_central_difference(ctx, cases):
    import oracle

    g = cases["rmat12"]
    rng = np.random.default_rng(9)
    w = np.exp(rng.standard_normal(g.E)).astype(np.float32)
    seed = _subset_seed(g.V, rng)
    _, gr, _ = _run(ctx, g, w, seed, **CONV)
    w64 = w.astype(np.float64)

    def loss(ww):
        r, _ = oracle.pagerank_weighted_f64(g.offsets, g.col, ww)
        return float(seed @ r)

    for trial in range(3):
        d = w64 * rng.standard_normal(g.E)  # relative perturbation keeps weights positive
        h = 1e-4
        fd = (loss(w64 + h * d) - loss(w64 - h * d)) / (2 * h)
        ana = float(np.dot(gr.astype(np.float64), d))
        assert abs(ana - fd) <= 1e-4 * abs(fd) + 1e-9, (trial, ana, fd)


def test_bit_reproducible(ctx, cases):
    g = cases["dangling"]
    rng = np.random.default_rng(1)
    w = np.exp(rng.standard_normal(g.E)).astype(np.float32)
    seed = rng.standard_normal(g.V)
    r1, g1, s1 = _run(ctx, g, w, seed, **CONV)
    r2, g2, s2 = _run(ctx, g, w, seed, **CONV)
    assert s1 == s2
    assert np.array_equal(r1.view(np.uint32), r2.view(np.uint32))
    assert np.array_equal(g1.view(np.uint32), g2.view(np.uint32))


def test_fixed_sweeps_and_unit_weights_match_plain_pagerank(ctx, cases):
    import oracle

    g = cases["dangling"]
    ones = np.ones(g.E, np.float32)
    r, _, (nf, na) = _run(ctx, g, ones, np.zeros(g.V), damping=0.85, total_rank=1.0, iterations=20, epsilon=0.0)
    assert (nf, na) == (20, 20)
    r64, n64 = oracle.pagerank_weighted_f64(g.offsets, g.col, ones.astype(np.float64), iterations=20, epsilon=0.0)
    assert n64 == 20
    assert (np.abs(r - r64) / r64).max() <= TOL
    # The plain pull kernel on the transposed CSR with out-degrees computes the same 20 sweeps.
    t_off, t_col, _ = dpg.csr_transpose_perm(g.V, g.offsets, g.col)
    gin = dpg.Graph(ctx, t_off, t_col[:g.E])
    r_plain = dpg.pagerank(ctx, gin, np.diff(g.offsets).astype(np.int32), damping=0.85, total_rank=1.0,
                           iterations=20)
    assert (np.abs(r - r_plain) / r64).max() <= TOL


def test_zero_seed_gives_zero_gradient(ctx, cases):
    g = cases["rmat12"]
    w = np.exp(np.random.default_rng(2).standard_normal(g.E)).astype(np.float32)
    _, gr, (_, na) = _run(ctx, g, w, np.zeros(g.V), **CONV)
    assert na == 1
    assert not gr.any()


def test_gradcheck_small_graph(ctx):
    import torch

    from smdp_gb300.autograd import weighted_pagerank

    g = dpg.rmat_csr(5, 4, seed=5, weights=False)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    rng = np.random.default_rng(3)
    w = torch.tensor(rng.uniform(0.5, 2.0, g.E), dtype=torch.float32, device="cuda", requires_grad=True)
    fn = lambda ww: weighted_pagerank(ctx, dg, ww, **CONV)  # noqa: E731
    assert torch.autograd.gradcheck(fn, (w,), eps=1e-2, atol=1e-3, rtol=3e-2, nondet_tol=0.0)


def test_rmat20_vs_fp64(ctx):
    """The configuration the gradient is specified on: R-MAT scale 20, lognormal(0,1) weights, loss =
    sum of r over a random 1% vertex subset, against the FP64 reference gradient."""
    g = dpg.rmat_csr(20, 16, seed=20, weights=False)
    rng = np.random.default_rng(20)
    w = np.exp(rng.standard_normal(g.E)).astype(np.float32)
    seed = _subset_seed(g.V, rng)
    r, gr, (nf, na) = _run(ctx, g, w, seed, **CONV)
    assert nf < 2000 and na < 2000
    assert abs(float(r.astype(np.float64).sum()) - 1.0) < 1e-4
    rows, bound = _check_vs_fp64(g, w, seed, r, gr)
    # Scaling a row's weights leaves r unchanged: sum over each row of w * dL/dw vanishes, up to
    # the rounding of each term, which is bounded by TOL * w * bound.
    wd = w.astype(np.float64)
    row_sum = np.bincount(rows, wd * gr, minlength=g.V)
    row_bound = np.bincount(rows, wd * bound, minlength=g.V)
    assert (np.abs(row_sum) <= TOL * row_bound + 1e-30).all()
