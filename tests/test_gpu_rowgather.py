"""GPU parity for the row gathers through the C ABI.

SpMV: csr_spmv_kernel (SpMV_kernel.cu:81-96). FP32 results against the FP64 oracle with
tolerance |y - y64| <= 1e-5 * sum_e |a_e x_col(e)| per row (the relative error the
conditioning of a mixed-sign dot product allows); with the reference's own initialisation
(data[e] = e%13 + 0.5, x[i] = i%17 + 0.5, SpMV_wrapper.cu:105-110) every partial sum is exact in FP32,
so the result must equal FP64 bit for bit.
PageRank: pull sweeps (pagerank_kernel.cu:95-120, pagerank_wrapper.cu:199-244) against FP64, max
relative error <= 1e-5, with the L1 error reported; the reference's own mode (d=0.5, total 1000,
start from 0, iterate until every |new-old| <= 1e-13) against its FP32 restatement."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg, load_golden

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _hub_graph():
    # Rows of degree 0, 1, 255, 256, 257, 3000 and 70000 (segments and both fix-up paths).
    V = 80000
    src, dst = [], []
    rng = np.random.default_rng(5)
    for r, d in [(3, 1), (10, 255), (11, 256), (12, 257), (20, 3000), (21, 70000), (22, 2047), (23, 2049)]:
        src += [r] * d
        dst += rng.integers(0, V, d).tolist()
    s2 = rng.integers(100, V, 200000)
    src += s2.tolist()
    dst += rng.integers(0, V, 200000).tolist()
    return dpg.csr_from_arcs(V, src, dst)


@pytest.fixture(scope="module")
def graphs():
    d = load_golden("data_test.json")
    return {
        "data_test": dpg.CSR(d["V"], d["E"], d["source"], np.array(d["offsets"], np.int32),
                             np.array(d["col"], np.int32), None),
        "rmat12": dpg.rmat_csr(12, 16, seed=12, weights=False),
        "rmat16": dpg.rmat_csr(16, 16, seed=16, weights=False),
        "hubs": _hub_graph(),
        "grid": dpg.grid_csr(50, 70, seed=3),
    }


def _spmv_check(ctx, orc, g, vals, x):
    dg = dpg.Graph(ctx, g.offsets, g.col)
    y = dpg.spmv(ctx, dg, vals, x)
    y64, ay = orc.spmv_f32in(g.offsets, g.col, vals, x)
    err = np.abs(y.astype(np.float64) - y64)
    assert np.all(err <= TOL * np.maximum(ay, np.finfo(np.float32).tiny)), float(np.max(err / np.maximum(ay, 1e-30)))
    return y


def test_spmv_reference_init_is_exact(ctx, orc, graphs):
    g = graphs["data_test"]
    vals = (np.arange(g.E) % 13 + 0.5).astype(np.float32)
    x = (np.arange(g.V) % 17 + 0.5).astype(np.float32)
    y = dpg.spmv(ctx, dpg.Graph(ctx, g.offsets, g.col), vals, x)
    y64 = orc.spmv_f64(g.offsets, g.col, vals.astype(np.float64), x.astype(np.float64))
    assert np.array_equal(y.astype(np.float64), y64)


@pytest.mark.parametrize("name", ["rmat12", "rmat16", "hubs", "grid"])
def test_spmv_within_tolerance(ctx, orc, graphs, name):
    g = graphs[name]
    rng = np.random.default_rng(1)
    vals = rng.uniform(np.nextafter(0, 1), 1.0, g.E).astype(np.float32)
    x = rng.uniform(-1.0, 1.0, g.V).astype(np.float32)
    _spmv_check(ctx, orc, g, vals, x)


def test_spmv_deterministic(ctx, graphs):
    g = graphs["hubs"]
    rng = np.random.default_rng(2)
    vals = rng.uniform(0, 1, g.E).astype(np.float32)
    x = rng.uniform(-1, 1, g.V).astype(np.float32)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    a = dpg.spmv(ctx, dg, vals, x)
    b = dpg.spmv(ctx, dg, vals, x)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_spmv_empty_rows_and_tiny_graphs(ctx):
    c = dpg.csr_from_arcs(5, [], [], None)
    y = dpg.spmv(ctx, dpg.Graph(ctx, c.offsets, c.col), np.zeros(0, np.float32), np.ones(5, np.float32))
    assert y.tolist() == [0.0] * 5
    c = dpg.csr_from_arcs(1, [0, 0], [0, 0], None)
    y = dpg.spmv(ctx, dpg.Graph(ctx, c.offsets, c.col), np.array([2, 3], np.float32), np.array([4], np.float32))
    assert y.tolist() == [20.0]


def _pr_inputs(g):
    in_off, in_col = dpg.csr_transpose(g.V, g.offsets, g.col)
    return in_off, in_col, dpg.out_degrees(g.offsets)


@pytest.mark.parametrize("name", ["rmat12", "rmat16", "hubs", "grid", "data_test"])
def test_pagerank_20_iterations_vs_fp64(ctx, orc, graphs, name):
    g = graphs[name]
    in_off, in_col, od = _pr_inputs(g)
    gi = dpg.Graph(ctx, in_off, in_col)
    r = dpg.pagerank(ctx, gi, od, damping=0.85, total_rank=1.0, iterations=20)
    r64, _ = orc.pagerank_f64(in_off, in_col, od, damping=0.85, total=1.0, iterations=20)
    rel = np.abs(r - r64) / r64
    assert rel.max() <= TOL, (float(rel.max()), float(np.abs(r - r64).sum()))
    assert ctx.last_stats().iterations == 20


def test_pagerank_deterministic_and_dev_api(ctx, graphs):
    import torch

    g = graphs["rmat16"]
    in_off, in_col, od = _pr_inputs(g)
    gi = dpg.Graph(ctx, in_off, in_col)
    a = dpg.pagerank(ctx, gi, od)
    dev = torch.device("cuda:0")
    odt = torch.from_numpy(od).to(dev)
    rt = torch.empty(g.V, dtype=torch.float32, device=dev)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        dpg.pagerank_dev(ctx, gi, odt.data_ptr(), rt.data_ptr())
        ctx.synchronize()
    finally:
        ctx.set_stream(None)
    assert np.array_equal(a.view(np.uint32), rt.cpu().numpy().view(np.uint32))


def test_pagerank_zero_iterations_returns_initial_vector(ctx, graphs):
    g = graphs["rmat12"]
    in_off, in_col, od = _pr_inputs(g)
    r = dpg.pagerank(ctx, dpg.Graph(ctx, in_off, in_col), od, iterations=0)
    assert np.all(r == np.float32(1.0 / g.V))


def test_pagerank_reference_mode_data_test(ctx, orc, graphs):
    # d = 0.5 (pagerank_wrapper.cu:7), total 1000 (pagerank.h:15), initial ranks 0 (wrapper.cu:115),
    # stop when no |rank - new| > 1e-13 (wrapper.cu:8, kernel.cu:72-81).
    g = graphs["data_test"]
    in_off, in_col, od = _pr_inputs(g)
    r = dpg.pagerank(ctx, dpg.Graph(ctx, in_off, in_col), od, damping=0.5, total_rank=1000.0, init_zero=True,
                     iterations=10000, epsilon=1e-13)
    rf, n = orc.pagerank_ref_f32(in_off, in_col, od)
    r64, _ = orc.pagerank_f64(in_off, in_col, od, damping=0.5, total=1000.0, init_zero=True, iterations=500,
                              epsilon=1e-15)
    assert np.max(np.abs(r - r64) / r64) <= TOL
    assert np.max(np.abs(r - rf) / rf) <= TOL
    assert ctx.last_stats().iterations < 10000


def test_one_shot_pagerank_host_call(ctx, orc, graphs):
    g = graphs["rmat12"]
    in_off, in_col, od = _pr_inputs(g)
    r = dpg.pagerank_host(ctx, in_off, in_col, od)
    r64, _ = orc.pagerank_f64(in_off, in_col, od)
    assert np.max(np.abs(r - r64) / r64) <= TOL


def _plan_counts(off, rows_per_range=2048, tile_items=256, hub_degree=255, small_segs=8):
    """The row plan's greedy tiling, restated: per range of rows, consecutive rows share a tile while
    their merge items (rows + nonzeros) fit in 256; a row above degree 255 is cut into 256-nonzero
    segments (a hub, fixed up per thread with <= 8 segments, else per warp)."""
    off = np.asarray(off, np.int64)
    V = len(off) - 1
    tiles = small = big = segs = 0
    for r0 in range(0, V, rows_per_range):
        cur_rows = cur_items = 0
        for r in range(r0, min(V, r0 + rows_per_range)):
            d = int(off[r + 1] - off[r])
            if d > hub_degree:
                if cur_rows:
                    tiles += 1
                cur_rows = cur_items = 0
                n = (d + tile_items - 1) // tile_items
                tiles += n
                segs += n
                small, big = (small + 1, big) if n <= small_segs else (small, big + 1)
                continue
            if cur_items + d + 1 > tile_items:
                tiles += 1
                cur_rows = cur_items = 0
            cur_rows += 1
            cur_items += d + 1
        if cur_rows:
            tiles += 1
    return {"tiles": tiles, "hubs_small": small, "hubs_big": big, "segments": segs}


@pytest.mark.parametrize("name", ["data_test", "rmat12", "rmat16", "hubs", "grid"])
def test_device_row_plan_matches_restated_greedy(ctx, graphs, name):
    # The plan is built on the device (count, scan and write passes); its counts must equal the
    # greedy tiling restated here, for the out-edge CSR (SpMV) and the in-edge CSR (PageRank).
    g = graphs[name]
    in_off, in_col, _ = _pr_inputs(g)
    for off, col in ((g.offsets, g.col), (in_off, in_col)):
        assert dpg.Graph(ctx, off, col).plan_info() == _plan_counts(off)


@pytest.mark.parametrize("name", ["rmat12", "hubs", "data_test"])
def test_one_shot_matches_graph_path_bitwise(ctx, graphs, name):
    # The one-shot call renames columns by the out-degree array while the columns upload; the graph
    # path renames them by a column histogram. Rows keep their nonzero order either way, so the
    # ranks are the same bits, also when the out-degrees disagree with the columns (the order then
    # differs from the histogram's).
    g = graphs[name]
    in_off, in_col, od = _pr_inputs(g)
    rng = np.random.default_rng(17)
    for outdeg in (od, rng.permutation(od).astype(np.int32)):
        one = dpg.pagerank_host(ctx, in_off, in_col, outdeg, iterations=20)
        two = dpg.pagerank(ctx, dpg.Graph(ctx, in_off, in_col), outdeg, iterations=20)
        assert np.array_equal(one.view(np.uint32), two.view(np.uint32))


def test_one_shot_rejects_bad_input(ctx, graphs):
    # The one-shot call checks columns and offsets on the device; the errors are the graph path's.
    g = graphs["rmat12"]
    in_off, in_col, od = _pr_inputs(g)
    for bad in (g.V, -1, 1 << 30):
        col = in_col.copy()
        col[len(col) // 2 + 3] = bad
        with pytest.raises(dpg.DpgError) as e:
            dpg.pagerank_host(ctx, in_off, col, od)
        assert e.value.status == dpg.ERR_INVALID_ARG
        assert "column index out of range" in str(e.value)
    dec = in_off.copy()
    dec[1000] = dec[1002] + 1  # offsets decrease at vertex 1000
    with pytest.raises(dpg.DpgError) as e:
        dpg.pagerank_host(ctx, dec, in_col, od)
    assert e.value.status == dpg.ERR_INVALID_ARG and "offsets decrease at vertex" in str(e.value)
    for off in (np.concatenate([in_off[:-1], [in_off[-1] - 1]]).astype(np.int32),
                np.concatenate([[1], in_off[1:]]).astype(np.int32)):
        with pytest.raises(dpg.DpgError) as e:
            dpg.pagerank_host(ctx, off, in_col, od)
        assert e.value.status == dpg.ERR_INVALID_ARG and "offsets must start at 0 and end at E" in str(e.value)
    # The context stays usable, and the next one-shot call is right.
    r = dpg.pagerank_host(ctx, in_off, in_col, od, iterations=20)
    ref = dpg.pagerank(ctx, dpg.Graph(ctx, in_off, in_col), od, iterations=20)
    assert np.array_equal(r.view(np.uint32), ref.view(np.uint32))


def test_spmv_pagerank_rmat22_full_size(ctx, orc):
    # R-MAT scale 22, edge factor 16; FP32 values uniform in (0,1], x uniform in [-1,1];
    # PageRank d = 0.85, 20 iterations, dangling mass spread uniformly.
    g = dpg.rmat_csr(22, 16, seed=22, weights=False)
    rng = np.random.default_rng(22)
    vals = (1.0 - rng.random(g.E, dtype=np.float32)).astype(np.float32)
    x = rng.uniform(-1.0, 1.0, g.V).astype(np.float32)
    _spmv_check(ctx, orc, g, vals, x)
    in_off, in_col, od = _pr_inputs(g)
    r = dpg.pagerank(ctx, dpg.Graph(ctx, in_off, in_col), od, iterations=20)
    r64, _ = orc.pagerank_f64(in_off, in_col, od, iterations=20)
    assert np.max(np.abs(r - r64) / r64) <= TOL
    one = dpg.pagerank_host(ctx, in_off, in_col, od, iterations=20)
    assert np.array_equal(one.view(np.uint32), r.view(np.uint32))


@pytest.mark.parametrize("name", ["rmat16", "hubs"])
def test_column_renaming_is_bit_identical(ctx, graphs, name):
    g = graphs[name]
    rng = np.random.default_rng(9)
    vals = rng.uniform(0, 1, g.E).astype(np.float32)
    x = rng.uniform(-1, 1, g.V).astype(np.float32)
    plain = dpg.Graph(ctx, g.offsets, g.col)
    plain.set_relabel(False)
    renamed = dpg.Graph(ctx, g.offsets, g.col)
    a = dpg.spmv(ctx, plain, vals, x)
    b = dpg.spmv(ctx, renamed, vals, x)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    in_off, in_col, od = _pr_inputs(g)
    gp = dpg.Graph(ctx, in_off, in_col)
    gp.set_relabel(False)
    gr = dpg.Graph(ctx, in_off, in_col)
    ra = dpg.pagerank(ctx, gp, od)
    rb = dpg.pagerank(ctx, gr, od)
    assert np.array_equal(ra.view(np.uint32), rb.view(np.uint32))
