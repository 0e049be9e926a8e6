"""The FP64 weighted-PageRank gradient oracle against central differences of its own forward map.

The weighted PageRank and its edge-weight gradient have no counterpart in the reference, so the
oracle is pinned by calculus instead: every arc's derivative, and directional derivatives, must
match central differences of the FP64 fixed point.
"""
import numpy as np
import pytest

import oracle


def _tiny_graph():
    # 12 vertices: two dangling (5 and 11), a self-loop, a duplicate arc, a hub.
    arcs = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 2), (2, 0), (2, 4), (3, 3), (3, 4), (4, 0), (4, 1), (4, 2),
            (4, 3), (4, 5), (4, 6), (4, 7), (6, 8), (7, 8), (8, 9), (9, 10), (10, 0), (10, 11), (6, 11)]
    V = 12
    arcs.sort(key=lambda a: a[0])
    src = np.array([a[0] for a in arcs])
    col = np.array([a[1] for a in arcs], np.int32)
    off = np.zeros(V + 1, np.int32)
    np.add.at(off, src + 1, 1)
    return V, np.cumsum(off).astype(np.int32), col


def _loss(off, col, w, seed, **kw):
    r, _ = oracle.pagerank_weighted_f64(off, col, w, epsilon=1e-15, **kw)
    return float(seed @ r)


@pytest.mark.parametrize("damping", [0.85, 0.5])
def test_every_arc_matches_central_difference(damping):
    V, off, col = _tiny_graph()
    rng = np.random.default_rng(3)
    w = np.exp(rng.standard_normal(col.shape[0]))
    seed = np.zeros(V)
    seed[[2, 8, 11]] = 1.0
    r, lam, g = oracle.pagerank_weighted_grad_f64(off, col, w, seed, damping=damping)
    assert abs(r.sum() - 1.0) < 1e-12
    for e in range(col.shape[0]):
        h = 1e-6 * w[e]
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd = (_loss(off, col, wp, seed, damping=damping) - _loss(off, col, wm, seed, damping=damping)) / (2 * h)
        assert abs(fd - g[e]) <= 1e-7 + 1e-5 * abs(fd), (e, fd, g[e])


def test_scale_invariance_per_row():
    # Row-normalised weights: scaling all of u's out-weights by a constant leaves r unchanged, so
    # the gradient is orthogonal to w within each row.
    V, off, col = _tiny_graph()
    rng = np.random.default_rng(4)
    w = np.exp(rng.standard_normal(col.shape[0]))
    seed = rng.standard_normal(V)
    _, _, g = oracle.pagerank_weighted_grad_f64(off, col, w, seed)
    for u in range(V):
        b, e = off[u], off[u + 1]
        if e > b:
            assert abs(np.dot(g[b:e], w[b:e])) < 1e-12
