"""The allocation-free SSSP entry point (dpg_sssp_noalloc_dev) against the regular one.

It serves callers that cannot allocate device memory: code inside a CUDA-graph capture and engines
that own the whole device pool. The test allocates its own inputs and output (the caller's job),
calls the entry point twice in a row through the C ABI (the second call must not see stale state
from the first), and requires distances identical to dpg_sssp's (integers: exact). This file is
collected last so a failure here cannot hide another test's result."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg

pytestmark = pytest.mark.gpu


def _device_inputs(torch, g):
    dev = torch.device("cuda", 0)
    off = torch.from_numpy(g.offsets).to(dev)
    pairs = torch.from_numpy(np.stack([g.col, g.weights], axis=1).astype(np.int32).copy()).to(dev)
    dist = torch.full((g.V,), -1, dtype=torch.int32, device=dev)
    return off, pairs, dist


def test_noalloc_matches_regular_sssp_on_two_calls():
    import torch

    g = dpg.rmat_csr(14, 16, seed=1, wmin=1, wmax=100)
    off, pairs, dist = _device_inputs(torch, g)
    deg = np.diff(g.offsets)
    sources = [0, int(np.argmax(deg))]
    with dpg.Context(0) as ctx:
        dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
        expected = [dpg.sssp(ctx, dg, s) for s in sources]
        dg.close()
    stream = torch.cuda.current_stream().cuda_stream
    for s, exp in zip(sources, expected):
        dpg.sssp_noalloc_dev(g.V, g.E, off.data_ptr(), pairs.data_ptr(), s, dist.data_ptr(), stream)
        torch.cuda.synchronize()
        assert np.array_equal(dist.cpu().numpy(), exp)
    assert not np.array_equal(expected[0], expected[1])


def test_noalloc_rejects_graphs_beyond_its_limit():
    import torch

    dev = torch.device("cuda", 0)
    off = torch.zeros(8, dtype=torch.int32, device=dev)
    pairs = torch.zeros(16, dtype=torch.int32, device=dev)
    dist = torch.zeros(8, dtype=torch.int32, device=dev)
    with pytest.raises(dpg.DpgError) as e:
        dpg.sssp_noalloc_dev(dpg.NOALLOC_MAX_VERTICES + 1, 0, off.data_ptr(), pairs.data_ptr(), 0, dist.data_ptr())
    assert e.value.status == dpg.ERR_CAPACITY and "no-alloc scratch limit" in str(e.value)
    with pytest.raises(dpg.DpgError) as e:
        dpg.sssp_noalloc_dev(7, dpg.NOALLOC_MAX_ARCS + 1, off.data_ptr(), pairs.data_ptr(), 0, dist.data_ptr())
    assert e.value.status == dpg.ERR_CAPACITY
