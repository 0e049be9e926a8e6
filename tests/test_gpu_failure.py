"""Failure detection without faulting the GPU: every wait of the persistent kernels is bounded.

The self test runs the grid barrier with one CTA missing, so the wait can only end by its time
limit; the kernel must record DPG_ERR_TIMEOUT in the device status word and return, leaving the
context usable for the next solve."""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu


def test_barrier_wait_times_out_and_context_survives(ctx, orc):
    t0 = time.time()
    status = dpg.selftest_barrier_timeout(ctx, 0.5)
    dt = time.time() - t0
    assert status == dpg.ERR_TIMEOUT
    assert dt < 20.0
    g = dpg.rmat_csr(10, 8, seed=1)
    dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
    assert np.array_equal(dpg.sssp(ctx, dg, 0), orc.sssp_dijkstra(g.offsets, g.col, g.weights, 0))


def test_selftest_rejects_unbounded_limits(ctx):
    assert dpg.selftest_barrier_timeout(ctx, 0.0) == dpg.ERR_INVALID_ARG
    assert dpg.selftest_barrier_timeout(ctx, 1000.0) == dpg.ERR_INVALID_ARG
