"""Batches of graphs through the C ABI: many graphs and many SSSP sources in one persistent launch,
one PageRank per graph in one gather per sweep, both captured as one CUDA graph.

SSSP distances must equal the plain single-graph solve (and Dijkstra) bit for bit; PageRank must
match the plain kernel on each graph alone and the FP64 oracle within 1e-5 relative; the captured
graph must reproduce the direct calls exactly, and autotuning must not change any result."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu
NSRC = 8
SWEEPS = 20


def _graphs():
    specs = dpg.rmat_batch_specs(22, seed=3, vmin=512, vmax=1 << 16)
    gs = dpg.rmat_batch(specs, seed=100)
    # Edge cases: a single vertex without arcs, a weighted path, a graph whose vertices are all
    # dangling but one.
    gs.append(dpg.csr_from_arcs(1, np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32)))
    gs.append(dpg.csr_from_arcs(5, [0, 1, 2, 3], [1, 2, 3, 4], [7, 1, 100, 3]))
    gs.append(dpg.csr_from_arcs(6, [2, 2, 2], [0, 1, 5], [1, 2, 3]))
    return gs


@pytest.fixture(scope="module")
def batch_case(ctx):
    gs = _graphs()
    rng = np.random.default_rng(8)
    src = np.stack([rng.integers(0, g.V, NSRC) for g in gs]).astype(np.int32)
    b = dpg.Batch(ctx, gs)
    return gs, src, b


def _device(n, dtype):
    import torch

    return torch.empty(n, dtype=dtype, device="cuda")


def test_union_layout(batch_case):
    gs, _, b = batch_case
    assert b.n == len(gs)
    assert b.V == sum(g.V for g in gs) and b.E == sum(g.E for g in gs)


def test_batch_sssp_equals_plain_per_graph(ctx, batch_case):
    import torch

    import oracle

    gs, src, b = batch_case
    dist = _device(NSRC * b.V, torch.int32)
    b.sssp_dev(src, dist.data_ptr())
    ctx.synchronize()
    d = dist.cpu().numpy().reshape(b.V, NSRC)  # vertex-major: d[v, k]
    for k, g in enumerate(gs):
        v0, v1 = int(b.vstart[k]), int(b.vstart[k + 1])
        dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
        for c in range(NSRC):
            plain = dpg.sssp(ctx, dg, int(src[k, c]))
            assert np.array_equal(d[v0:v1, c], plain), (k, c)
        exact = oracle.sssp_dijkstra(g.offsets, g.col, g.weights, int(src[k, 0]))
        assert np.array_equal(d[v0:v1, 0], exact), k


@pytest.mark.parametrize("nsrc", [1, 3, 4, 12, 32])
def test_batch_sssp_other_source_counts(ctx, batch_case, nsrc):
    import torch

    import oracle

    gs, _, b = batch_case
    rng = np.random.default_rng(nsrc)
    src = np.stack([rng.integers(0, g.V, nsrc) for g in gs]).astype(np.int32)
    src[0, :] = src[0, 0]  # repeated sources in one graph share a vertex's mask
    dist = _device(nsrc * b.V, torch.int32)
    b.sssp_dev(src, dist.data_ptr())
    ctx.synchronize()
    d = dist.cpu().numpy().reshape(b.V, nsrc)
    for k in (0, 5, len(gs) - 2, len(gs) - 1):
        g = gs[k]
        v0, v1 = int(b.vstart[k]), int(b.vstart[k + 1])
        for c in range(nsrc):
            exact = oracle.sssp_dijkstra(g.offsets, g.col, g.weights, int(src[k, c]))
            assert np.array_equal(d[v0:v1, c], exact), (k, c)


def test_batch_sssp_unaligned_labels(ctx, batch_case):
    """Labels that do not start on a 16-byte boundary take the source-by-source relaxation; the
    distances equal the aligned run's (which reads eight labels at a time)."""
    import torch

    gs, src, b = batch_case
    aligned = _device(NSRC * b.V, torch.int32)
    b.sssp_dev(src, aligned.data_ptr())
    buf = _device(NSRC * b.V + 1, torch.int32)
    buf.fill_(-5)
    b.sssp_dev(src, buf.data_ptr() + 4)
    ctx.synchronize()
    assert int(buf[0]) == -5
    assert torch.equal(buf[1:], aligned)


def test_batch_pagerank_equals_plain_and_fp64(ctx, batch_case):
    import torch

    import oracle

    gs, _, b = batch_case
    rank = _device(b.V, torch.float32)
    b.pagerank_dev(rank.data_ptr(), damping=0.85, total_rank=1.0, iterations=SWEEPS)
    ctx.synchronize()
    r = rank.cpu().numpy()
    for k, g in enumerate(gs):
        v0, v1 = int(b.vstart[k]), int(b.vstart[k + 1])
        in_off, in_col = dpg.csr_transpose(g.V, g.offsets, g.col)
        od = np.diff(g.offsets).astype(np.int32)
        plain = dpg.pagerank(ctx, dpg.Graph(ctx, in_off, in_col), od, damping=0.85, total_rank=1.0,
                             iterations=SWEEPS)
        r64, _ = oracle.pagerank_f64(in_off, in_col, od, damping=0.85, total=1.0, iterations=SWEEPS)
        assert np.abs(r[v0:v1] - plain).max() <= 1e-5 * r64.max(), k
        rel = np.abs(r[v0:v1] - r64) / r64
        assert rel.max() <= 1e-5, (k, rel.max())
        assert abs(r[v0:v1].astype(np.float64).sum() - 1.0) < 1e-4


def test_captured_graph_reproduces_direct_calls(ctx, batch_case):
    import torch

    gs, src, b = batch_case
    d1, r1 = _device(NSRC * b.V, torch.int32), _device(b.V, torch.float32)
    b.sssp_dev(src, d1.data_ptr())
    b.pagerank_dev(r1.data_ptr(), iterations=SWEEPS)
    ctx.synchronize()
    d2, r2 = _device(NSRC * b.V, torch.int32), _device(b.V, torch.float32)
    # Capture, replays, and replays on the legacy default stream (which cannot be captured itself).
    for stream in (None, None, 0, 0, None):
        ctx.set_stream(stream)
        d2.fill_(-1)
        r2.fill_(-1)
        torch.cuda.synchronize()
        b.run(src, d2.data_ptr(), r2.data_ptr(), pr_opts_={"iterations": SWEEPS})
        ctx.synchronize()
        assert torch.equal(d1, d2)
        assert torch.equal(r1.view(torch.int32), r2.view(torch.int32))
    ctx.set_stream(None)
    assert b.launches() == 3 + 3 + 3 * SWEEPS


def test_autotune_picks_a_candidate_and_changes_nothing(ctx, batch_case):
    import torch

    gs, src, b = batch_case
    d1, r1 = _device(NSRC * b.V, torch.int32), _device(b.V, torch.float32)
    b.run(src, d1.data_ptr(), r1.data_ptr(), pr_opts_={"iterations": SWEEPS})
    ctx.synchronize()
    saved = b.tuning
    t = b.autotune(src)
    assert t["hub_threshold"] in (16, 32, 64, 128) and t["chunk"] in (128, 256, 512)
    assert t["pr_hot"] in (0, 4096, 16384, -1)
    assert b.tuning == t
    d2, r2 = _device(NSRC * b.V, torch.int32), _device(b.V, torch.float32)
    for tune in (t, {"hub_threshold": 1, "chunk": 128, "pr_hot": 0}, {"hub_threshold": 100000, "chunk": 512, "pr_hot": -1}):
        b.tuning = tune
        b.run(src, d2.data_ptr(), r2.data_ptr(), pr_opts_={"iterations": SWEEPS})
        ctx.synchronize()
        assert torch.equal(d1, d2), tune
        assert torch.equal(r1.view(torch.int32), r2.view(torch.int32)), tune
    b.tuning = saved


def test_per_graph_tuning_changes_nothing(ctx, batch_case):
    """Mixed per-graph SSSP settings run as one launch per setting; the distances (and the captured
    graph's replays) equal those of one batch-wide setting, and the batch-wide setter drops them."""
    import torch

    gs, src, b = batch_case
    d1, r1 = _device(NSRC * b.V, torch.int32), _device(b.V, torch.float32)
    b.run(src, d1.data_ptr(), r1.data_ptr(), pr_opts_={"iterations": SWEEPS})
    ctx.synchronize()
    saved = b.tuning
    rng = np.random.default_rng(11)
    hub = rng.choice([1, 16, 64, 128, 100000], b.n).astype(np.int32)
    chunk = rng.choice([128, 256, 512], b.n).astype(np.int32)
    b.set_graph_tuning(hub, chunk)
    t = b.graph_tuning()
    assert np.array_equal(t["hub_threshold"], hub) and np.array_equal(t["chunk"], chunk)
    groups = len(set(zip(hub.tolist(), chunk.tolist())))
    assert groups > 1
    d2, r2 = _device(NSRC * b.V, torch.int32), _device(b.V, torch.float32)
    d2.fill_(-1)
    b.sssp_dev(src, d2.data_ptr())
    ctx.synchronize()
    assert torch.equal(d1, d2)
    for _ in range(2):  # capture, then replay
        d2.fill_(-1)
        b.run(src, d2.data_ptr(), r2.data_ptr(), pr_opts_={"iterations": SWEEPS})
        ctx.synchronize()
        assert torch.equal(d1, d2)
        assert torch.equal(r1.view(torch.int32), r2.view(torch.int32))
    assert b.launches() == 3 * groups + 3 + 3 * SWEEPS
    bad = chunk.copy()
    bad[2] = 100
    with pytest.raises(dpg.DpgError):
        b.set_graph_tuning(hub, bad)
    b.tuning = saved  # the batch-wide setter applies to every graph again
    t = b.graph_tuning()
    assert np.all(t["hub_threshold"] == saved["hub_threshold"]) and np.all(t["chunk"] == saved["chunk"])


def test_autotune_chooses_per_size_class(ctx, batch_case):
    gs, src, b = batch_case
    saved = b.tuning
    b.autotune(src)
    t = b.graph_tuning()
    arcs = np.array([g.E for g in gs])
    cls = np.where(arcs < (1 << 17), 0, np.where(arcs < (1 << 21), 1, 2))
    for c in np.unique(cls):
        sel = cls == c
        assert len(set(t["hub_threshold"][sel].tolist())) == 1 and len(set(t["chunk"][sel].tolist())) == 1
    assert set(t["hub_threshold"].tolist()) <= {16, 32, 64, 128}
    assert set(t["chunk"].tolist()) <= {128, 256, 512}
    b.tuning = saved


def test_batch_rejects_bad_input(ctx, batch_case):
    import torch

    gs, src, b = batch_case
    dist, rank = _device(NSRC * b.V, torch.int32), _device(b.V, torch.float32)
    bad = src.copy()
    bad[3, 2] = gs[3].V
    with pytest.raises(dpg.DpgError):
        b.sssp_dev(bad, dist.data_ptr())
    with pytest.raises(dpg.DpgError):
        b.pagerank_dev(rank.data_ptr(), epsilon=1e-6)
    # An arc that leaves its graph's vertex range.
    g0 = dpg.csr_from_arcs(3, [0, 1], [1, 2], [1, 1])
    g1 = dpg.csr_from_arcs(3, [0], [1], [1])
    leaking = g0._replace(col=np.array([1, 4], np.int32))  # vertex 4 of the union is graph 1's
    with pytest.raises(dpg.DpgError):
        dpg.Batch(ctx, [leaking, g1])
