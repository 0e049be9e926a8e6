"""Recursive BFS with device-side child launches (CDP2): the reference's naive, warp-, block- and
grid-consolidated recursive traversals, kept as a measured comparison.

Levels must equal the oracle's BFS exactly whenever the call succeeds; a traversal that needs more
nesting generations than the device allows must come back as an error, never as wrong levels."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu
VARIANTS = [dpg.CDP_NAIVE, dpg.CDP_WARP, dpg.CDP_BLOCK, dpg.CDP_GRID]


def _levels(ctx, g, src, variant):
    import torch

    lv = torch.empty(g.V, dtype=torch.int32, device="cuda")
    dg = dpg.Graph(ctx, g.offsets, g.col)
    st = dpg.bfs_cdp_dev(ctx, dg, src, variant, lv.data_ptr())
    return lv.cpu().numpy(), st


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("scale", [8, 12])
def test_cdp_levels_equal_oracle(ctx, variant, scale):
    import oracle

    g = dpg.rmat_csr(scale, 8, seed=scale, weights=False)
    deg = np.diff(g.offsets)
    src = int(np.flatnonzero(deg > 0)[0])
    lv, st = _levels(ctx, g, src, variant)
    assert st["failed_launches"] == 0
    assert st["launches"] >= 1
    assert np.array_equal(lv, oracle.bfs(g.offsets, g.col, src))


def test_cdp_matches_persistent_bfs(ctx):
    g = dpg.rmat_csr(14, 16, seed=14, weights=False)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    src = int(np.argmax(np.diff(g.offsets)))
    ref = dpg.bfs(ctx, dg, src)
    for variant in (dpg.CDP_BLOCK, dpg.CDP_GRID):
        lv, _ = _levels(ctx, g, src, variant)
        assert np.array_equal(lv, ref), variant


def test_cdp_too_deep_is_an_error_not_wrong_levels(ctx):
    # A 40-vertex path needs 39 generations of child launches; the device allows 24.
    n = 40
    g = dpg.csr_from_arcs(n, np.arange(n - 1), np.arange(1, n))
    for variant in VARIANTS:
        with pytest.raises(dpg.DpgError) as ei:
            _levels(ctx, g, 0, variant)
        assert "DPG_ERR_CAPACITY" in str(ei.value)
    # The context stays usable.
    g2 = dpg.rmat_csr(8, 8, seed=8, weights=False)
    lv, st = _levels(ctx, g2, int(np.flatnonzero(np.diff(g2.offsets))[0]), dpg.CDP_GRID)
    assert st["failed_launches"] == 0
