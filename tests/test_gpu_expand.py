"""GPU parity for the frontier expansion (SSSP and BFS) through the C ABI.

Integer results must be bit-exact: SSSP against Dijkstra (the unique fixed point of the
reference's relaxation, sssp_kernel.cu:40-61), BFS against bfs_cpu (bfs_rec.cpp:102-121), for every
work-mapping (the reference's -s 0..4 and the binned default) and degree thresholds. At full size
(R-MAT scale 24, 4096x4096 grid) the check is a certificate instead: d[src] = 0, no arc can
still relax, and every reached vertex has a tight in-arc; BFS levels are compared with the
all-cores CPU restatement and, on the grid, with the Manhattan distance."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg, load_golden

pytestmark = pytest.mark.gpu

SOLUTIONS = [dpg.SOL_THREAD, dpg.SOL_NAIVE, dpg.SOL_WARP, dpg.SOL_BLOCK, dpg.SOL_GRID, dpg.SOL_BINNED,
             dpg.SOL_DIROPT, dpg.SOL_NEARFAR]
DATA_TEST_DIST = [6853, 8841, 12973, 11908, 5652, 1741, 48923, 0, 16618, 3910, 2320, 61857, 55633, 17426, 19168,
                  10230, 15116, 17185, 16866, 23257]
DATA_TEST_LEVEL = [3, 4, 4, 3, 2, 1, 2, 0, 1, 2, 1, 4, 3, 2, 3, 3, 4, 5, 5, 4]


def _star_plus_chain():
    # Hub 0 with 5000 out-arcs (grid-wide chunks), a 2000-vertex chain hanging off it (many
    # iterations), back arcs, a self-loop and duplicate arcs.
    V = 7001
    src, dst, w = [], [], []
    for i in range(1, 5001):
        src.append(0); dst.append(i); w.append(1 + i % 17)
    for i in range(5000, 7000):
        src.append(i); dst.append(i + 1); w.append(3)
    for i in range(1, 5001, 7):
        src.append(i); dst.append(0); w.append(2)
    src += [5, 5, 5, 9]; dst += [6, 6, 5, 9]; w += [1, 0, 4, 0]
    return dpg.csr_from_arcs(V, src, dst, w)


def _zero_weight_random(seed):
    rng = np.random.default_rng(seed)
    V, E = 3000, 20000
    return dpg.csr_from_arcs(V, rng.integers(0, V, E), rng.integers(0, V, E), rng.integers(0, 4, E))


@pytest.fixture(scope="module")
def graphs():
    d = load_golden("data_test.json")
    return {
        "data_test": (dpg.CSR(d["V"], d["E"], d["source"], np.array(d["offsets"], np.int32),
                              np.array(d["col"], np.int32), np.array(d["weights"], np.int32)), d["source"]),
        "rmat10": (dpg.rmat_csr(10, 8, seed=3, wmin=1, wmax=100), 0),
        # The single-GPU parity workload: R-MAT scale 14, edge factor 16, weights [1,100], source 0.
        "rmat14": (dpg.rmat_csr(14, 16, seed=1, wmin=1, wmax=100), 0),
        "star_chain": (_star_plus_chain(), 0),
        "grid64": (dpg.grid_csr(64, 64, seed=2, wmin=1, wmax=1000), 0),
        "zero_w": (_zero_weight_random(4), 17),
        "rmat12_unpermuted": (dpg.rmat_csr(12, 16, seed=8, wmin=1, wmax=255, permute=False), 0),
    }


@pytest.fixture(scope="module")
def devgraphs(ctx, graphs):
    return {k: dpg.Graph(ctx, g.offsets, g.col, g.weights) for k, (g, _) in graphs.items()}


@pytest.mark.parametrize("sol", SOLUTIONS)
def test_sssp_data_test_known_answer(ctx, devgraphs, sol):
    d = dpg.sssp(ctx, devgraphs["data_test"], 7, solution=sol)
    assert d.tolist() == DATA_TEST_DIST


@pytest.mark.parametrize("sol", SOLUTIONS)
def test_bfs_data_test_known_answer(ctx, devgraphs, sol):
    lv = dpg.bfs(ctx, devgraphs["data_test"], 7, solution=sol)
    assert lv.tolist() == DATA_TEST_LEVEL


@pytest.mark.parametrize("name", ["rmat10", "rmat14", "star_chain", "grid64", "zero_w", "rmat12_unpermuted"])
@pytest.mark.parametrize("sol", SOLUTIONS)
def test_sssp_bit_exact_vs_dijkstra(ctx, orc, graphs, devgraphs, name, sol):
    g, s = graphs[name]
    expect = orc.sssp_dijkstra(g.offsets, g.col, g.weights, s)
    got = dpg.sssp(ctx, devgraphs[name], s, solution=sol)
    assert np.array_equal(got, expect)


@pytest.mark.parametrize("name", ["rmat10", "rmat14", "star_chain", "grid64", "zero_w", "rmat12_unpermuted"])
@pytest.mark.parametrize("sol", SOLUTIONS)
def test_bfs_bit_exact_vs_bfs_cpu(ctx, orc, graphs, devgraphs, name, sol):
    g, s = graphs[name]
    expect = orc.bfs(g.offsets, g.col, s)
    got = dpg.bfs(ctx, devgraphs[name], s, solution=sol)
    assert np.array_equal(got, expect)


@pytest.mark.parametrize("threshold,hub", [(1, 1), (2, 32), (16, 64), (64, 256), (1000, 100000)])
@pytest.mark.parametrize("sol", [dpg.SOL_WARP, dpg.SOL_BLOCK, dpg.SOL_GRID, dpg.SOL_BINNED, dpg.SOL_DIROPT,
                                 dpg.SOL_NEARFAR])
def test_thresholds(ctx, orc, graphs, devgraphs, threshold, hub, sol):
    g, s = graphs["rmat14"]
    expect = orc.sssp_dijkstra(g.offsets, g.col, g.weights, s)
    got = dpg.sssp(ctx, devgraphs["rmat14"], s, solution=sol, threshold=threshold, hub_threshold=hub)
    assert np.array_equal(got, expect)
    lv = dpg.bfs(ctx, devgraphs["rmat14"], s, solution=sol, threshold=threshold, hub_threshold=hub)
    assert np.array_equal(lv, orc.bfs(g.offsets, g.col, s))


def test_many_sources_and_repeat_calls(ctx, orc, graphs, devgraphs):
    g, _ = graphs["rmat14"]
    rng = np.random.default_rng(0)
    deg = np.diff(g.offsets)
    for s in rng.choice(np.flatnonzero(deg > 0), 6, replace=False).tolist() + [int(np.argmax(deg))]:
        expect = orc.sssp_dijkstra(g.offsets, g.col, g.weights, s)
        for _ in range(2):
            assert np.array_equal(dpg.sssp(ctx, devgraphs["rmat14"], s), expect)
        assert np.array_equal(dpg.bfs(ctx, devgraphs["rmat14"], s), orc.bfs(g.offsets, g.col, s))


def test_stats_report_work(ctx, graphs, devgraphs):
    g, s = graphs["rmat14"]
    dpg.sssp(ctx, devgraphs["rmat14"], s)
    st = ctx.last_stats()
    assert st.iterations >= 2 and st.edges_scanned >= 0.5 * g.E and st.grid_blocks >= 152


def test_wide_graphs_run_the_4_cta_build(ctx, graphs, devgraphs):
    """Graphs with hubs (R-MAT) run the binned SSSP and direction-optimizing BFS with 4 CTAs per
    SM; a hubless graph of at most 8 arcs per vertex (the 64 x 64 grid) with 3. Distances and
    levels are exact either way (the other tests of this file)."""
    sms = ctx.sm_count
    for name, per_sm in (("rmat14", 4), ("grid64", 3)):
        g, s = graphs[name]
        for solve in (dpg.sssp, dpg.bfs):
            solve(ctx, devgraphs[name], s, solution=dpg.SOL_BINNED if solve is dpg.sssp else dpg.SOL_DIROPT)
            assert ctx.last_stats().grid_blocks == per_sm * sms, (name, solve.__name__)


def test_single_vertex_and_isolated_source(ctx):
    g = dpg.Graph(ctx, np.array([0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert dpg.sssp(ctx, g, 0).tolist() == [0]
    assert dpg.bfs(ctx, g, 0).tolist() == [0]
    c = dpg.csr_from_arcs(4, [1, 2], [2, 3], [5, 6])
    g2 = dpg.Graph(ctx, c.offsets, c.col, c.weights)
    assert dpg.sssp(ctx, g2, 0).tolist() == [0, dpg.INF_COST, dpg.INF_COST, dpg.INF_COST]
    assert dpg.bfs(ctx, g2, 1).tolist() == [dpg.UNDEFINED_LEVEL, 0, 1, 2]


def test_inf_semantics_match_reference_int_relaxation(ctx, orc):
    big = (1 << 30) - 10
    c = dpg.csr_from_arcs(4, [0, 1, 2], [1, 2, 3], [big, 20, 5])
    g = dpg.Graph(ctx, c.offsets, c.col, c.weights)
    for sol in SOLUTIONS:
        assert dpg.sssp(ctx, g, 0, solution=sol).tolist() == [0, big, dpg.INF_COST, dpg.INF_COST]


def test_invalid_arguments(ctx, devgraphs):
    g = devgraphs["data_test"]
    with pytest.raises(dpg.DpgError) as e:
        dpg.sssp(ctx, g, 20)
    assert e.value.status == dpg.ERR_INVALID_ARG
    with pytest.raises(dpg.DpgError) as e:
        dpg.sssp(ctx, g, 0, solution=9)
    assert e.value.status == dpg.ERR_INVALID_ARG
    c = dpg.csr_from_arcs(3, [0], [1], [1])
    unweighted = dpg.Graph(ctx, c.offsets, c.col)
    with pytest.raises(dpg.DpgError) as e:
        dpg.sssp(ctx, unweighted, 0)
    assert e.value.status == dpg.ERR_INVALID_ARG
    with pytest.raises(dpg.DpgError) as e:
        dpg.Graph(ctx, c.offsets, c.col, np.array([-1], np.int32))
    assert e.value.status == dpg.ERR_INVALID_ARG
    with pytest.raises(dpg.DpgError) as e:
        dpg.Graph(ctx, np.array([0, 1, 1, 1], np.int32), np.array([7], np.int32))
    assert e.value.status == dpg.ERR_INVALID_ARG
    # The context stays usable after rejected calls.
    assert dpg.sssp(ctx, g, 7).tolist() == DATA_TEST_DIST


def test_iteration_cap_reports_capacity(ctx, graphs, devgraphs):
    with pytest.raises(dpg.DpgError) as e:
        dpg.sssp(ctx, devgraphs["star_chain"], 0, max_iterations=3)
    assert e.value.status == dpg.ERR_CAPACITY
    g, s = graphs["star_chain"]
    assert dpg.sssp(ctx, devgraphs["star_chain"], 0)[7000] > 0


def test_device_pointer_api_with_torch_stream(ctx, orc, graphs):
    import torch

    g, s = graphs["rmat14"]
    dev = torch.device("cuda:0")
    off = torch.from_numpy(g.offsets).to(dev)
    col = torch.from_numpy(g.col).to(dev)
    w = torch.from_numpy(g.weights).to(dev)
    dg = dpg.Graph.from_device(ctx, g.V, g.E, off.data_ptr(), col.data_ptr(), w.data_ptr())
    dist = torch.empty(g.V, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    try:
        dpg.sssp_dev(ctx, dg, s, dist.data_ptr())
        ctx.synchronize()
    finally:
        ctx.set_stream(None)
    assert np.array_equal(dist.cpu().numpy(), orc.sssp_dijkstra(g.offsets, g.col, g.weights, s))


def test_one_shot_host_call(ctx, orc, graphs):
    g, s = graphs["rmat10"]
    got = dpg.sssp_host(ctx, g.offsets, g.col, g.weights, s)
    assert np.array_equal(got, orc.sssp_dijkstra(g.offsets, g.col, g.weights, s))


# ------------------------------------------------------------------------------- full size -------
def _certificate(off, col, w, dist, src):
    """Exact SSSP certificate on the GPU (torch used as plumbing only)."""
    import torch

    dev = torch.device("cuda:0")
    offt = torch.from_numpy(off).to(dev)
    colt = torch.from_numpy(col).to(dev).long()
    wt = torch.from_numpy(w).to(dev).long()
    d = torch.from_numpy(dist).to(dev).long()
    V = off.shape[0] - 1
    deg = (offt[1:] - offt[:-1]).long()
    u = torch.repeat_interleave(torch.arange(V, device=dev), deg)
    du = d[u]
    dv = d[colt]
    cand = du + wt
    finite = du < dpg.INF_COST
    violated = finite & (cand < dpg.INF_COST) & (dv > cand)
    tight = finite & (cand == dv)
    has_tight = torch.zeros(V, dtype=torch.bool, device=dev)
    has_tight[colt[tight]] = True
    reached = d < dpg.INF_COST
    reached[src] = False
    ok = int(d[src]) == 0 and not bool(violated.any()) and bool(has_tight[reached].all())
    return ok, int(reached.sum()) + 1


@pytest.fixture(scope="module")
def rmat24():
    # R-MAT scale 24, edge factor 16, weights uniform in [1,255].
    return dpg.rmat_csr(24, 16, seed=24, wmin=1, wmax=255)


def test_sssp_bfs_rmat24_full_size(ctx, orc, rmat24):
    g = rmat24
    dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
    deg = np.diff(g.offsets)
    rng = np.random.default_rng(24)
    sources = [int(s) for s in rng.choice(np.flatnonzero(deg > 0), 2, replace=False)]
    for s in sources:
        dist = dpg.sssp(ctx, dg, s)
        ok, reached = _certificate(g.offsets, g.col, g.weights, dist, s)
        assert ok and reached > g.V // 4
        lv = dpg.bfs(ctx, dg, s)
        assert np.array_equal(lv, orc.bfs_omp(g.offsets, g.col, s))
        assert np.array_equal(dpg.bfs(ctx, dg, s, solution=dpg.SOL_DIROPT), lv)
    # The reference's consolidation mappings and near-far at full size too (one source).
    for sol in (dpg.SOL_WARP, dpg.SOL_BLOCK, dpg.SOL_GRID, dpg.SOL_NEARFAR):
        d2 = dpg.sssp(ctx, dg, sources[0], solution=sol)
        assert np.array_equal(d2, dpg.sssp(ctx, dg, sources[0]))


def test_sssp_bfs_grid4096_full_size(ctx):
    n = 4096
    g = dpg.grid_csr(n, n, seed=4096, wmin=1, wmax=1000)
    assert g.E == 67092480
    dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
    s = int(np.random.default_rng(1).integers(0, g.V))
    dist = dpg.sssp(ctx, dg, s)
    ok, reached = _certificate(g.offsets, g.col, g.weights, dist, s)
    assert ok and reached == g.V
    assert np.array_equal(dpg.sssp(ctx, dg, s, solution=dpg.SOL_NEARFAR), dist)
    lv = dpg.bfs(ctx, dg, s)
    r, c = np.divmod(np.arange(g.V), n)
    assert np.array_equal(lv, np.abs(r - s // n) + np.abs(c - s % n))
    assert np.array_equal(dpg.bfs(ctx, dg, s, solution=dpg.SOL_DIROPT), lv)


@pytest.mark.parametrize("delta", [1, 7, 100, 10**9])
def test_nearfar_any_step_gives_exact_distances(ctx, orc, delta):
    g = dpg.rmat_csr(12, 16, seed=12, wmin=1, wmax=255)
    dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
    s = int(np.argmax(np.diff(g.offsets)))
    exact = orc.sssp_dijkstra(g.offsets, g.col, g.weights, s)
    assert np.array_equal(dpg.sssp(ctx, dg, s, solution=dpg.SOL_NEARFAR, delta=delta), exact)
    # Zero-weight arcs and distances landing exactly on a threshold.
    z = dpg.csr_from_arcs(6, [0, 1, 2, 3, 4, 0], [1, 2, 3, 4, 5, 5], [0, delta % 1000, 0, 0, delta % 1000, 999])
    dz = dpg.Graph(ctx, z.offsets, z.col, z.weights)
    assert np.array_equal(dpg.sssp(ctx, dz, 0, solution=dpg.SOL_NEARFAR, delta=delta),
                          orc.sssp_dijkstra(z.offsets, z.col, z.weights, 0))
