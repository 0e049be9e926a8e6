"""The allocation-free SSSP entry point (dpg_sssp_noalloc_dev) against the regular one.

It serves callers that must not allocate device memory: engines that reserve the whole device pool
for their own arena, and plugin hosts that hand out only buffers they own. The tests allocate the
inputs and the output themselves (the caller's job), call the entry point through the C ABI twice
in a row (the second call must not see stale state from the first), and require distances
identical to dpg_sssp's and to the oracle's Dijkstra (integers: exact). This file is collected
last so a failure here cannot hide another test's result."""
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


def _check_two_calls(torch, orc, g, sources):
    off, pairs, dist = _device_inputs(torch, g)
    with dpg.Context(0) as ctx:
        dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
        expected = [dpg.sssp(ctx, dg, s) for s in sources]
        dg.close()
    stream = torch.cuda.current_stream().cuda_stream
    for s, exp in zip(sources, expected):
        assert np.array_equal(exp, orc.sssp_dijkstra(g.offsets, g.col, g.weights, s))
        dpg.sssp_noalloc_dev(g.V, g.E, off.data_ptr(), pairs.data_ptr(), s, dist.data_ptr(), stream)
        torch.cuda.synchronize()
        assert np.array_equal(dist.cpu().numpy(), exp)
    assert not np.array_equal(expected[0], expected[1])


def test_noalloc_matches_regular_sssp_on_two_calls(orc):
    import torch

    g = dpg.rmat_csr(14, 16, seed=1, wmin=1, wmax=100)
    deg = np.diff(g.offsets)
    _check_two_calls(torch, orc, g, [0, int(np.argmax(deg))])


def test_noalloc_at_its_size_limit_with_hubs(orc):
    """V and E exactly at the limits, with hub rows above the 1024-arc chunking degree, so the
    chunk lists of the scratch layout fill."""
    import torch

    g = dpg.rmat_csr(18, 16, seed=18, wmin=1, wmax=255)
    assert (g.V, g.E) == (dpg.NOALLOC_MAX_VERTICES, dpg.NOALLOC_MAX_ARCS)
    deg = np.diff(g.offsets)
    assert int((deg >= 1024).sum()) >= 8
    rng = np.random.default_rng(18)
    _check_two_calls(torch, orc, g, [int(np.argmax(deg))] + [int(s) for s in rng.choice(np.flatnonzero(deg > 0), 1)])


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


def test_noalloc_rejects_bad_graphs_before_relaxing(orc):
    """A neighbour id outside [0, V), a negative weight or falling offsets: DPG_ERR_INVALID_ARG from
    the device check, the distances untouched, and the next good call exact again."""
    import torch

    g = dpg.rmat_csr(10, 8, seed=4, wmin=1, wmax=100)
    off, pairs, dist = _device_inputs(torch, g)
    src = int(np.argmax(np.diff(g.offsets)))
    bad_pairs = pairs.clone()
    bad_pairs[5, 0] = g.V + 3
    neg_pairs = pairs.clone()
    neg_pairs[9, 1] = -2
    bad_off = off.clone()
    bad_off[4] = bad_off[6] + 1
    for o, p, what in ((off, bad_pairs, "neighbour id"), (off, neg_pairs, "weight"), (bad_off, pairs, "offsets")):
        dist.fill_(-7)
        with pytest.raises(dpg.DpgError) as e:
            dpg.sssp_noalloc_dev(g.V, g.E, o.data_ptr(), p.data_ptr(), src, dist.data_ptr())
        assert e.value.status == dpg.ERR_INVALID_ARG and what in str(e.value)
        assert bool((dist == -7).all())
    dpg.sssp_noalloc_dev(g.V, g.E, off.data_ptr(), pairs.data_ptr(), src, dist.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(dist.cpu().numpy(), orc.sssp_dijkstra(g.offsets, g.col, g.weights, src))
