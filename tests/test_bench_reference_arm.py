"""bench.py's reference arm: the CPU PageRank over a graph the oracle generates, without loading
the GPU implementation's library, and printing the same config as the GPU arm."""
from __future__ import annotations

import json
import subprocess
import sys

from conftest import ROOT

PROBE = r"""
import argparse, json, sys
sys.path.insert(0, {root!r})
import bench
bench.SCALE = 10
bench.run_reference(argparse.Namespace(steps=1, warmup=0), 1, 0)
maps = open('/proc/self/maps').read()
print(json.dumps({{"libdpg_mapped": 'libdpg' in maps}}))
"""


def test_reference_arm_loads_no_gpu_library_and_prints_the_shared_config():
    out = subprocess.run([sys.executable, "-c", PROBE.format(root=str(ROOT))], capture_output=True, text=True,
                         timeout=300, cwd=str(ROOT))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[1]
    assert probe == {"libdpg_mapped": False}
    sys.path.insert(0, str(ROOT))
    import bench

    assert line["impl"] == "reference"
    assert line["config"] == bench.bench_config(1, 1 << 10, 16 << 10)
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_oracle_generator_equals_library_generator(orc):
    from conftest import dpg
    import numpy as np

    for scale, ef, seed, weights in ((9, 16, 22, False), (11, 8, 5, True)):
        off, col, w = orc.rmat_csr(scale, ef, seed, wmin=1, wmax=255, weights=weights)
        g = dpg.rmat_csr(scale, ef, seed=seed, wmin=1, wmax=255, weights=weights)
        assert np.array_equal(off, g.offsets) and np.array_equal(col, g.col)
        if weights:
            assert np.array_equal(w, g.weights)
        a, b = orc.csr_transpose(off, col)
        c, d = dpg.csr_transpose(g.V, g.offsets, g.col)
        assert np.array_equal(a, c) and np.array_equal(b, d)
