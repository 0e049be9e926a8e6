"""Command-line apps (gpu-sssp, gpu-bfs-rec, gpu-SpMV, gpu-pg): the reference apps' flags,
messages and exit codes (apps/sssp/src/sssp.cpp:51-188 and siblings). CPU-only checks here; the
GPU runs are in test_gpu_apps.py."""
from __future__ import annotations

import subprocess

import pytest

from conftest import dpg, load_golden

BIN = dpg.PKG_DIR / "bin"
APPS = ["gpu-sssp", "gpu-bfs-rec", "gpu-SpMV", "gpu-pg", "gpu-graph-color"]


def run(app, *args):
    return subprocess.run([str(BIN / app), *map(str, args)], capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("app", APPS)
def test_usage_without_arguments_and_with_h(app):
    for args in ([], ["-h"], ["--help"]):
        r = run(app, *args)
        assert r.returncode == 0
        assert "Usage:" in r.stderr and "--import,-i" in r.stderr


@pytest.mark.parametrize("app", APPS)
def test_missing_file_is_reported_like_the_reference(app, tmp_path):
    r = run(app, "-i", tmp_path / "missing.gr")
    assert r.returncode == 1 and "Error: NULL file pointer." in r.stderr
    assert "CONFIGURATION:" in r.stderr and "- Graph file:" in r.stderr


@pytest.mark.parametrize("app", APPS)
def test_malformed_file_exits_with_error(app, tmp_path):
    p = tmp_path / "bad.gr"
    p.write_text("p sp 3 5\na 1 2 3\n")
    r = run(app, "-i", p)
    assert r.returncode == 2 and "Error:" in r.stderr


def test_no_device_is_an_error_not_a_cpu_fallback(tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rec = load_golden("data_test.json")
    p = tmp_path / "d.gr"
    a = rec["arcs"]
    dpg.write_dimacs9(p, rec["V"], a["src"], a["dst"], a["w"], source=rec["source"])
    for app in APPS:
        r = run(app, "-i", p, "-v")
        assert r.returncode == 1 and "DPG_ERR_NO_DEVICE" in r.stdout


def test_cache_flag_writes_and_reuses_a_binary_csr(tmp_path):
    import os
    import time

    import numpy as np

    rec = load_golden("data_test.json")
    p = tmp_path / "d.gr"
    a = rec["arcs"]
    dpg.write_dimacs9(p, rec["V"], a["src"], a["dst"], a["w"], source=rec["source"])
    cache = tmp_path / "d.gr.dpgcsr"
    run("gpu-sssp", "-i", p, "--cache")  # the graph is loaded (and cached) before any device work
    assert cache.exists()
    g, h = dpg.read_graph(p), dpg.read_graph_cache(cache)
    assert np.array_equal(g.offsets, h.offsets) and np.array_equal(g.col, h.col)
    assert np.array_equal(g.weights, h.weights) and g.source == h.source
    # A cache older than the input is rebuilt.
    old = time.time() - 100
    os.utime(cache, (old, old))
    run("gpu-sssp", "-i", p, "--cache")
    assert cache.stat().st_mtime > old + 50
