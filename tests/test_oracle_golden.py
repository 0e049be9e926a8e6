"""Pins the CPU oracle against the reference: its only dataset and known answers, its own bfs_cpu
output (recorded in tests/golden by make_golden.py), and, where the reference tree is present, the
reference's host code run live."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import dpg, load_golden

# Known answers for datasets/data_test.gr from source `s 8` (0-based vertex 7).
DATA_TEST_DIST = [6853, 8841, 12973, 11908, 5652, 1741, 48923, 0, 16618, 3910, 2320, 61857, 55633, 17426, 19168,
                  10230, 15116, 17185, 16866, 23257]
DATA_TEST_LEVEL = [3, 4, 4, 3, 2, 1, 2, 0, 1, 2, 1, 4, 3, 2, 3, 3, 4, 5, 5, 4]
DATA_TEST_OUTDEG = [2, 1, 1, 2, 3, 3, 2, 3, 2, 2, 2, 1, 2, 3, 2, 3, 3, 1, 1, 1]
DATA_TEST_COLOR = [1, 2, 1, 2, 3, 4, 5, 5, 6, 1, 6, 1, 6, 7, 8, 8, 9, 10, 10, 9]


@pytest.fixture(scope="module")
def data_test():
    return load_golden("data_test.json")


def test_data_test_fixture_shape(data_test):
    assert data_test["V"] == 20 and data_test["E"] == 40 and data_test["source"] == 7
    assert np.diff(data_test["offsets"]).tolist() == DATA_TEST_OUTDEG


def test_sssp_dijkstra_known_answer(orc, data_test):
    d = orc.sssp_dijkstra(data_test["offsets"], data_test["col"], data_test["weights"], data_test["source"])
    assert d.tolist() == DATA_TEST_DIST


def test_sssp_worklist_matches_dijkstra(orc, data_test):
    d, passes = orc.sssp_worklist(data_test["offsets"], data_test["col"], data_test["weights"], data_test["source"])
    assert d.tolist() == DATA_TEST_DIST and passes >= 1


def test_bfs_known_answer_and_reference_bfs_cpu(orc, data_test):
    lv = orc.bfs(data_test["offsets"], data_test["col"], data_test["source"])
    assert lv.tolist() == DATA_TEST_LEVEL
    assert lv.tolist() == data_test["bfs_levels"]  # recorded from the reference's bfs_cpu


def test_color_known_answer(orc, data_test):
    c, rounds = orc.color(data_test["offsets"], data_test["col"])
    assert c.tolist() == DATA_TEST_COLOR
    assert rounds == max(DATA_TEST_COLOR) + 1  # the last round colours nothing and stops the loop


def test_bfs_reference_on_rmat_fixture(orc):
    r = load_golden("rmat_s8.json")
    lv = orc.bfs(r["offsets"], r["col"], 0)
    assert lv.tolist() == r["bfs_levels"]


def _random_graph(rng, V, E, wmax=50):
    src = rng.integers(0, V, E).astype(np.int32)
    dst = rng.integers(0, V, E).astype(np.int32)
    w = rng.integers(0, wmax + 1, E).astype(np.int32)
    return dpg.csr_from_arcs(V, src, dst, w)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_dijkstra_equals_reference_schedule_fixed_point(orc, seed):
    rng = np.random.default_rng(seed)
    g = _random_graph(rng, 300, 1500)
    d1 = orc.sssp_dijkstra(g.offsets, g.col, g.weights, 0)
    d2, _ = orc.sssp_worklist(g.offsets, g.col, g.weights, 0)
    d3 = orc.sssp_bf_omp(g.offsets, g.col, g.weights, 0)
    assert np.array_equal(d1, d2) and np.array_equal(d1, d3)


def test_bf_omp_repeated_runs_stay_exact(orc):
    """The OpenMP Bellman-Ford (the timed CPU baseline) run many times: its queued flag is cleared
    and its distance read with sequentially consistent accesses, so an improvement made while a
    vertex is being popped is never lost (with a relaxed clear, about 1 run in 200 of this fixture
    came out wrong)."""
    graphs = []
    for seed in range(4):
        g = _random_graph(np.random.default_rng(seed), 300, 1500)
        graphs.append((g, orc.sssp_dijkstra(g.offsets, g.col, g.weights, 0)))
    threads = max(4, os.cpu_count() or 4)  # explicit: an earlier call may have left OpenMP at 1 thread
    for rep in range(150):
        g, want = graphs[rep % 4]
        assert np.array_equal(orc.sssp_bf_omp(g.offsets, g.col, g.weights, 0, threads=threads), want), rep


def test_dijkstra_inf_semantics(orc):
    # A chain whose total reaches 2^30: the int relaxation never lowers an INF label with it.
    big = (1 << 30) - 10
    g = dpg.csr_from_arcs(4, [0, 1, 2], [1, 2, 3], [big, 20, 5])
    d = orc.sssp_dijkstra(g.offsets, g.col, g.weights, 0)
    d2, _ = orc.sssp_worklist(g.offsets, g.col, g.weights, 0)
    assert d.tolist() == [0, big, orc.INF, orc.INF] == d2.tolist()


@pytest.mark.parametrize("seed", [5, 6])
def test_bfs_omp_equals_bfs_cpu(orc, seed):
    rng = np.random.default_rng(seed)
    g = _random_graph(rng, 500, 2000)
    assert np.array_equal(orc.bfs(g.offsets, g.col, 3), orc.bfs_omp(g.offsets, g.col, 3))


def test_spmv_reference_known_answer_mode(orc, data_test):
    # SpMV_wrapper.cu:100-110 initialises data[e] = e%13 + 0.5 and x[i] = i%17 + 0.5 (FP64).
    E, V = data_test["E"], data_test["V"]
    data = np.arange(E) % 13 + 0.5
    x = np.arange(V) % 17 + 0.5
    y = orc.spmv_f64(data_test["offsets"], data_test["col"], data, x)
    off, col = np.array(data_test["offsets"]), np.array(data_test["col"])
    expect = [sum(data[e] * x[col[e]] for e in range(off[r], off[r + 1])) for r in range(V)]
    assert np.allclose(y, expect, rtol=0, atol=1e-12)


def test_pagerank_oracles_agree(orc):
    g = dpg.rmat_csr(8, 8, seed=11)
    in_off, in_col = dpg.csr_transpose(g.V, g.offsets, g.col)
    od = dpg.out_degrees(g.offsets)
    r64, n = orc.pagerank_f64(in_off, in_col, od, damping=0.85, total=1.0, iterations=20)
    assert n == 20 and abs(r64.sum() - 1.0) < 1e-12  # dangling mass redistributed: total conserved
    r32 = orc.pagerank_omp_f32(in_off, in_col, od, damping=0.85, total=1.0, iterations=20)
    assert np.max(np.abs(r32 - r64) / r64) < 1e-5


def test_pagerank_reference_mode_converges_to_f64_fixed_point(orc, data_test):
    od = np.diff(data_test["offsets"]).astype(np.int32)
    in_off, in_col = data_test["in_offsets"], data_test["in_col"]
    rf, n = orc.pagerank_ref_f32(in_off, in_col, od, damping=0.5, total=1000.0, init_zero=True,
                                 max_iterations=10000, epsilon=1e-13)
    r64, _ = orc.pagerank_f64(in_off, in_col, od, damping=0.5, total=1000.0, init_zero=True, iterations=200,
                              epsilon=1e-15)
    assert n < 10000
    assert np.max(np.abs(rf - r64) / r64) < 1e-5
    assert abs(r64.sum() - 1000.0) < 1e-9


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference host code not built here")
def test_live_reference_loader_equals_fixture(orc, data_test):
    from pathlib import Path
    V, E, s, off, col, w, in_off, in_col = orc.ref_load(Path(orc.REFERENCE_TREE) / "datasets" / "data_test.gr")
    assert (V, E, s) == (data_test["V"], data_test["E"], data_test["source"])
    assert off.tolist() == data_test["offsets"] and col.tolist() == data_test["col"]
    assert w.tolist() == data_test["weights"] and in_col.tolist() == data_test["in_col"]
    lv = orc.ref_bfs_cpu(s, V)
    assert lv.tolist() == orc.bfs(off, col, s).tolist()


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference host code not built here")
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_live_reference_bfs_cpu_on_generated_graphs(orc, tmp_path, seed):
    s, d, w = dpg.rmat_arcs(10, 6 * 1024, seed=seed)
    p = tmp_path / "g.gr"
    dpg.write_dimacs9(p, 1024, s, d, w, source=5)
    V, E, src, off, col, ww, in_off, in_col = orc.ref_load(p)
    g = dpg.read_graph(p)
    assert np.array_equal(g.offsets, off) and np.array_equal(g.col, col) and np.array_equal(g.weights, ww)
    assert src == 5 == g.source
    assert np.array_equal(orc.ref_bfs_cpu(src, V), orc.bfs(off, col, src))
