"""GPU colouring (dpg_color) against the reference's round rule (graph_color_kernel.cu:28-49,
graph_color_wrapper.cu:113-130), restated by the oracle; integers, so bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg, load_golden

pytestmark = pytest.mark.gpu
DATA_TEST_COLOR = [1, 2, 1, 2, 3, 4, 5, 5, 6, 1, 6, 1, 6, 7, 8, 8, 9, 10, 10, 9]


def test_color_data_test_known_answer(ctx):
    d = load_golden("data_test.json")
    g = dpg.Graph(ctx, d["offsets"], d["col"])
    assert dpg.color(ctx, g).tolist() == DATA_TEST_COLOR


@pytest.mark.parametrize("maker", ["rmat12", "rmat16_unpermuted", "grid", "random_dups", "star"])
def test_color_bit_exact_vs_oracle(ctx, orc, maker):
    if maker == "rmat12":
        c = dpg.rmat_csr(12, 16, seed=5, weights=False)
    elif maker == "rmat16_unpermuted":
        c = dpg.rmat_csr(16, 8, seed=6, weights=False, permute=False)
    elif maker == "grid":
        c = dpg.grid_csr(40, 60, seed=1)
    elif maker == "random_dups":
        rng = np.random.default_rng(3)
        s = rng.integers(0, 2000, 30000)
        c = dpg.csr_from_arcs(2000, np.concatenate([s, s[:500], [7, 7]]),
                              np.concatenate([rng.integers(0, 2000, 30000), rng.integers(0, 2000, 500), [7, 3]]))
    else:  # one vertex with 5000 lower neighbours and every other vertex pointing at the hub
        V = 6000
        src = [5999] * 5000 + list(range(5999))
        dst = list(range(5000)) + [5999] * 5999
        c = dpg.csr_from_arcs(V, src, dst)
    g = dpg.Graph(ctx, c.offsets, c.col)
    expect, rounds = orc.color(c.offsets, c.col)
    got = dpg.color(ctx, g)
    assert np.array_equal(got, expect)
    assert int(got.max()) == rounds - 1


def test_color_empty_and_single(ctx):
    c = dpg.csr_from_arcs(3, [], [], None)
    assert dpg.color(ctx, dpg.Graph(ctx, c.offsets, c.col)).tolist() == [1, 1, 1]
