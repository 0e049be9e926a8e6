"""Parity against the reference's own kernels.

tests/golden/refgpu.npz holds the outputs of the reference's kernels (sssp_kernel.cu,
graph_color_kernel.cu, SpMV_kernel.cu, pagerank_kernel.cu), compiled from its tree and run on a
GB300 by tests/golden/make_golden_gpu.py, on the reference's datasets/data_test.gr and on seeded
R-MAT graphs (scale 14 for SSSP and colouring, scale 12 for SpMV and PageRank).

CPU tests pin the oracle to those outputs bit for bit. GPU tests pin the CUDA path to them:
distances and colours exactly, SpMV within 1e-5 of each row's sum of |terms| of the reference's
FP64 result, and PageRank within 1e-5 relative of FP64 plus the reference's own FP32 distance from
FP64 of the reference's FP32 result.
"""
from __future__ import annotations

import sys

import numpy as np
import pytest

from conftest import GOLDEN, dpg

sys.path.insert(0, str(GOLDEN))
import make_golden_gpu as mg  # noqa: E402

TOL = 1e-5


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLDEN / "refgpu.npz")


@pytest.fixture(scope="module")
def graphs():
    gs, _ = mg.graphs()
    return gs


# ------------------------------------------------------------------------ oracle (CPU) ----
def test_oracle_sssp_equals_reference_kernels(orc, ref, graphs):
    for name in ("data_test", "rmat14"):
        off, col, w, _, _ = graphs[name]
        for i, s in enumerate(ref[f"{name}/sssp_sources"]):
            exp = ref[f"{name}/sssp_dist"][i]
            assert np.array_equal(orc.sssp_dijkstra(off, col, w, int(s)), exp), (name, s)
            d, _ = orc.sssp_worklist(off, col, w, int(s))
            assert np.array_equal(d, exp), (name, s)


def test_oracle_color_equals_reference_kernel(orc, ref, graphs):
    for name in ("data_test", "rmat14"):
        off, col, _, _, _ = graphs[name]
        c, rounds = orc.color(off, col)
        assert np.array_equal(c, ref[f"{name}/color"]) and rounds == int(ref[f"{name}/color_rounds"])


def test_oracle_spmv_equals_reference_kernel_bitwise(orc, ref, graphs):
    for name in ("data_test", "rmat12"):
        off, col, _, _, _ = graphs[name]
        V, E = off.shape[0] - 1, col.shape[0]
        for mode, (data, x) in (("refvals", mg.spmv_reference_inputs(E, V)), ("f32vals", mg.spmv_random_inputs(E, V))):
            y = orc.spmv_f64(off, col, np.asarray(data, np.float64), np.asarray(x, np.float64))
            assert np.array_equal(y, ref[f"{name}/spmv_{mode}_y"]), (name, mode)


def test_oracle_pagerank_equals_reference_kernels_bitwise(orc, ref, graphs):
    for name in ("data_test", "rmat12"):
        off, _, _, in_off, in_col = graphs[name]
        od = np.diff(off).astype(np.int32)
        r, n = orc.pagerank_ref_f32(in_off, in_col, od, damping=0.5, total=1000.0, init_zero=True,
                                    max_iterations=100000, epsilon=1e-13)
        assert np.array_equal(r, ref[f"{name}/pagerank_refmode_rank"])
        assert n == int(ref[f"{name}/pagerank_refmode_sweeps"])
        r, n = orc.pagerank_ref_f32(in_off, in_col, od, damping=0.85, total=1.0, init_zero=False, max_iterations=20,
                                    epsilon=-1.0)
        assert np.array_equal(r, ref[f"{name}/pagerank_d085_rank"]) and n == 20


def test_fixture_graphs_are_the_library_and_loader_graphs(orc, graphs):
    """The R-MAT inputs of the fixtures, built by the oracle, are the library's graphs (same
    generator, convertCSR and invertGraph order), and the data_test arrays are the reference
    loader's (recorded by make_golden.py)."""
    off, col, w, in_off, in_col = graphs["rmat14"]
    g = dpg.rmat_csr(mg.RMAT14["scale"], mg.RMAT14["edge_factor"], seed=mg.RMAT14["seed"], wmin=mg.RMAT14["wmin"],
                     wmax=mg.RMAT14["wmax"])
    assert np.array_equal(off, g.offsets) and np.array_equal(col, g.col) and np.array_equal(w, g.weights)
    t_off, t_col = dpg.csr_transpose(g.V, g.offsets, g.col)
    assert np.array_equal(in_off, t_off) and np.array_equal(in_col, t_col)
    dt = mg.json.loads((GOLDEN / "data_test.json").read_text())
    assert graphs["data_test"][0].tolist() == dt["offsets"] and graphs["data_test"][4].tolist() == dt["in_col"]


# ------------------------------------------------------------------------ CUDA path (GPU) ----
@pytest.mark.gpu
def test_sssp_equals_reference_kernels_every_mapping(ctx, ref, graphs):
    for name in ("data_test", "rmat14"):
        off, col, w, _, _ = graphs[name]
        g = dpg.Graph(ctx, off, col, w)
        for i, s in enumerate(ref[f"{name}/sssp_sources"]):
            exp = ref[f"{name}/sssp_dist"][i]
            for sol in range(8):
                assert np.array_equal(dpg.sssp(ctx, g, int(s), solution=sol), exp), (name, s, sol)


@pytest.mark.gpu
def test_color_equals_reference_kernel(ctx, ref, graphs):
    for name in ("data_test", "rmat14"):
        off, col, _, _, _ = graphs[name]
        c = dpg.color(ctx, dpg.Graph(ctx, off, col))
        assert np.array_equal(c, ref[f"{name}/color"]), name


@pytest.mark.gpu
def test_spmv_against_reference_kernel_fp64(ctx, orc, ref, graphs):
    for name in ("data_test", "rmat12"):
        off, col, _, _, _ = graphs[name]
        V, E = off.shape[0] - 1, col.shape[0]
        g = dpg.Graph(ctx, off, col)
        # The app's own values: every product and partial sum is a multiple of 1/4 below 2^22, exact in
        # FP32, so the FP32 result equals the reference's FP64 one.
        data, x = mg.spmv_reference_inputs(E, V)
        y = dpg.spmv(ctx, g, np.asarray(data, np.float32), np.asarray(x, np.float32))
        assert np.array_equal(y.astype(np.float64), ref[f"{name}/spmv_refvals_y"])
        vals, x = mg.spmv_random_inputs(E, V)
        y = dpg.spmv(ctx, g, vals, x)
        _, bound = orc.spmv_f32in(off, col, vals, x)
        assert np.all(np.abs(y - ref[f"{name}/spmv_f32vals_y"]) <= TOL * np.maximum(bound, 1e-30)), name


@pytest.mark.gpu
def test_pagerank_against_reference_kernels(ctx, orc, ref, graphs):
    for name in ("data_test", "rmat12"):
        off, _, _, in_off, in_col = graphs[name]
        od = np.diff(off).astype(np.int32)
        gi = dpg.Graph(ctx, in_off, in_col)
        for key, opts, f64 in (
                ("pagerank_d085_rank", dict(damping=0.85, total_rank=1.0, iterations=20),
                 dict(damping=0.85, total=1.0, iterations=20)),
                ("pagerank_refmode_rank", dict(damping=0.5, total_rank=1000.0, init_zero=True, iterations=100000,
                                               epsilon=1e-13),
                 dict(damping=0.5, total=1000.0, init_zero=True, iterations=500, epsilon=1e-15))):
            r = dpg.pagerank(ctx, gi, od, **opts)
            r_ref = ref[f"{name}/{key}"]
            r64, _ = orc.pagerank_f64(in_off, in_col, od, **f64)
            ref_err = float(np.max(np.abs(r_ref - r64) / r64))
            assert np.max(np.abs(r - r64) / r64) <= TOL, (name, key)
            assert np.max(np.abs(r - r_ref) / r_ref) <= TOL + ref_err, (name, key, ref_err)
