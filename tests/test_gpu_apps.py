"""The command-line apps on the GPU, on the reference's own dataset (datasets/data_test.gr, rebuilt
from tests/golden/data_test.json): outputs must match the reference's formats and answers."""
from __future__ import annotations

import re
import subprocess

import numpy as np
import pytest

from conftest import dpg, load_golden

pytestmark = pytest.mark.gpu
BIN = dpg.PKG_DIR / "bin"
DATA_TEST_DIST = [6853, 8841, 12973, 11908, 5652, 1741, 48923, 0, 16618, 3910, 2320, 61857, 55633, 17426, 19168,
                  10230, 15116, 17185, 16866, 23257]


@pytest.fixture(scope="module")
def gr(tmp_path_factory):
    rec = load_golden("data_test.json")
    p = tmp_path_factory.mktemp("apps") / "data_test.gr"
    a = rec["arcs"]
    dpg.write_dimacs9(p, rec["V"], a["src"], a["dst"], a["w"], source=rec["source"])
    return p


def run(app, *args):
    return subprocess.run([str(BIN / app), *map(str, args)], capture_output=True, text=True, timeout=300)


@pytest.mark.parametrize("sol", range(6))
def test_gpu_sssp_debug_output_is_outputcost(gr, sol):
    r = run("gpu-sssp", "-i", gr, "-d", "-v", "-s", sol, "--verify")
    assert r.returncode == 0, r.stdout + r.stderr
    expect = "".join(f"From Node 8 -> {i + 1} is {d}\n" for i, d in enumerate(DATA_TEST_DIST))
    assert expect in r.stdout
    assert "PASS: GPU sssp !" in r.stdout
    for label in ("CUDA runtime initialization:", "CUDA kernel execution:", "CUDA D2H cudaMemcpy:"):
        assert label in r.stdout
    assert "Source node is: 8" in r.stderr and "Iteration:" in r.stderr


def test_gpu_sssp_out_file_and_source_flag(gr, tmp_path):
    out = tmp_path / "cost.txt"
    r = run("gpu-sssp", "-i", gr, "--out", out)
    assert r.returncode == 0
    assert out.read_text() == "".join(f"From Node 8 -> {i + 1} is {d}\n" for i, d in enumerate(DATA_TEST_DIST))
    r = run("gpu-sssp", "-i", gr, "--source", 1, "--verify")
    assert r.returncode == 0 and "PASS" in r.stdout


@pytest.mark.parametrize("sol", range(7))
def test_gpu_bfs_rec_validates_like_the_reference(gr, sol):
    r = run("gpu-bfs-rec", "-i", gr, "-s", sol, "-v")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "===MAIN=== :: [num_nodes,num_edges] = 20, 40" in r.stdout
    assert "PASS: GPU bfs rec !" in r.stdout
    assert "===MAIN=== :: CUDA kernel execution:" in r.stdout


def test_gpu_spmv_debug_output_matches_fp64(gr):
    r = run("gpu-SpMV", "-i", gr, "-d", "--verify")
    assert r.returncode == 0 and "PASS: GPU SpMV !" in r.stdout
    rec = load_golden("data_test.json")
    off, col = np.array(rec["offsets"]), np.array(rec["col"])
    data = np.arange(rec["E"]) % 13 + 0.5
    x = np.arange(rec["V"]) % 17 + 0.5
    ys = [float(m) for m in re.findall(r"y\[\d+\] = ([-0-9.]+)", r.stderr)]
    expect = [sum(data[e] * x[col[e]] for e in range(off[i], off[i + 1])) for i in range(rec["V"])]
    assert ys == [float(f"{v:f}") for v in expect]


def test_gpu_pagerank_reference_mode(gr, tmp_path, orc):
    out = tmp_path / "rank.txt"
    r = run("gpu-pg", "-i", gr, "-d", "--out", out)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PageRank ends in" in r.stderr
    got = np.array([float(m) for m in re.findall(r"Node \d+: ([0-9.]+)", out.read_text())])
    rec = load_golden("data_test.json")
    od = np.diff(rec["offsets"]).astype(np.int32)
    ref, _ = orc.pagerank_ref_f32(rec["in_offsets"], rec["in_col"], od)
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-6)


def test_gpu_graph_color_matches_reference_rule(gr):
    r = run("gpu-graph-color", "-i", gr, "-d")
    assert r.returncode == 0, r.stdout + r.stderr
    expect = [1, 2, 1, 2, 3, 4, 5, 5, 6, 1, 6, 1, 6, 7, 8, 8, 9, 10, 10, 9]
    assert "".join(f"Node {i + 1}: {c}\n" for i, c in enumerate(expect)) in r.stdout
    assert "Execution time:" in r.stderr
