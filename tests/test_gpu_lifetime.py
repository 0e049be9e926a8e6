"""Object lifetimes across the C ABI: graphs and batches may outlive the context they were created on.

Destroying a context orphans its graphs and batches; destroying them afterwards frees their device
memory without touching the context, and any solve on them is rejected."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu


def test_graph_and_batch_outlive_their_context(ctx):
    c2 = dpg.Context(0)
    g = dpg.rmat_csr(8, 8, seed=1)
    dg = dpg.Graph(c2, g.offsets, g.col, g.weights)
    b = dpg.Batch(c2, [g, g])
    d = dpg.sssp(c2, dg, 0)
    assert d[0] == 0
    c2.close()
    # The orphans cannot be used with any context, and free cleanly.
    with pytest.raises(dpg.DpgError):
        dpg.sssp(ctx, dg, 0)
    dg.close()
    b.close()
    # The session context is unaffected.
    dg2 = dpg.Graph(ctx, g.offsets, g.col, g.weights)
    assert np.array_equal(dpg.sssp(ctx, dg2, 0), d)
