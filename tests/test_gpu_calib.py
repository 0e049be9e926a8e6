"""The random-read ceiling measurement (dpg_calibrate_random_reads): positive, and reads from a
16 MB array (L2-resident) at least as fast as from a 1 GB one (mostly HBM)."""
from __future__ import annotations

import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu


def test_random_read_ceiling(ctx):
    l2 = dpg.calibrate_random_reads(ctx, 4 << 20, iters=50)
    hbm = dpg.calibrate_random_reads(ctx, 1 << 28, iters=20)
    assert l2 > 1e10 and hbm > 1e9
    assert l2 >= hbm
    with pytest.raises(dpg.DpgError):
        dpg.calibrate_random_reads(ctx, 10, iters=1)


def test_hot_cache_counts(ctx):
    """The arcs served by the gather's shared-memory hot cache: all of them when every arc points at
    one column, none with the renaming off, and between 0 and E on an R-MAT graph, where the most
    gathered columns come first."""
    import numpy as np

    star = dpg.csr_from_arcs(1000, np.arange(1, 1000), np.zeros(999, np.int64))
    gs = dpg.Graph(ctx, star.offsets, star.col)
    hc = gs.hot_cache()
    assert hc["hot_entries"] >= 1 and hc["hot_arcs"] == star.E
    g = dpg.rmat_csr(14, 16, seed=3, weights=False)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    hc = dg.hot_cache()
    assert hc["hot_entries"] == min(g.V, hc["hot_entries"]) and 0 < hc["hot_arcs"] <= g.E
    counts = np.sort(np.bincount(g.col, minlength=g.V))[::-1]
    assert hc["hot_arcs"] <= int(counts[:hc["hot_entries"]].sum())  # the top columns bound it
    dg.set_relabel(False)
    assert dg.hot_cache() == {"hot_entries": 0, "hot_arcs": 0}
