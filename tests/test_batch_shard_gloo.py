"""Multi-rank batched workload on CPU (gloo, world size 2): graphs sharded by LPT on arcs x tasks
with no exchange step, each rank solving its own graphs, results gathered on rank 0.

Each rank computes the partition on its own; rank 0 checks that every rank computed the same
owners, that every graph was solved exactly once, that the gathered results equal one process
solving everything (oracle SSSP and FP64 PageRank stand in for the device solves), and that the
LPT loads stay within the list-scheduling bound."""
from __future__ import annotations

import os

import numpy as np
import pytest

NSRC, SWEEPS, NGRAPHS, SEED = 2, 5, 24, 77


def _solve(dpg, oracle, spec, k):
    g = dpg.rmat_batch([spec], seed=SEED * 1000 + k)[0]
    rng = np.random.default_rng(k)
    src = rng.integers(0, g.V, NSRC)
    dist = [oracle.sssp_dijkstra(g.offsets, g.col, g.weights, int(s)) for s in src]
    in_off, in_col = dpg.csr_transpose(g.V, g.offsets, g.col)
    r, _ = oracle.pagerank_f64(in_off, in_col, np.diff(g.offsets).astype(np.int32), iterations=SWEEPS)
    return k, np.stack(dist), r


def _rank_main(rank, world, store_path, out_path):
    import sys

    import torch.distributed as dist

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    from conftest import dpg
    import oracle

    # A file rendezvous in the test's temporary directory: no port to race for.
    dist.init_process_group("gloo", init_method=f"file://{store_path}", rank=rank, world_size=world)
    specs = dpg.rmat_batch_specs(NGRAPHS, seed=SEED, vmin=64, vmax=4096)
    cost = np.array([v * ef * (NSRC + SWEEPS) for v, ef in specs], np.int64)
    owner, load = dpg.partition_lpt(cost, world)
    mine = [_solve(dpg, oracle, specs[k], k) for k in range(NGRAPHS) if owner[k] == rank]
    gathered = [None] * world if rank == 0 else None
    dist.gather_object((rank, owner.tolist(), load.tolist(), mine), gathered, dst=0)
    if rank == 0:
        import pickle

        with open(out_path, "wb") as f:
            pickle.dump(gathered, f)
    dist.barrier()
    dist.destroy_process_group()


def test_lpt_partition_properties():
    from conftest import dpg

    rng = np.random.default_rng(3)
    cost = rng.integers(1, 10**9, 200)
    for parts in (1, 2, 3, 8):
        owner, load = dpg.partition_lpt(cost, parts)
        assert owner.min() >= 0 and owner.max() < parts
        assert np.array_equal(np.bincount(owner, cost, minlength=parts).astype(np.int64), load)
        assert load.max() <= cost.sum() / parts + cost.max()
        assert np.array_equal(owner, dpg.partition_lpt(cost, parts)[0])  # deterministic
    owner, load = dpg.partition_lpt(np.zeros(0, np.int64), 4)
    assert owner.size == 0 and not load.any()
    with pytest.raises(dpg.DpgError):
        dpg.partition_lpt([1, -1], 2)


def test_two_rank_sharded_batch_matches_one_process(tmp_path):
    import pickle

    import torch.multiprocessing as mp

    from conftest import dpg
    import oracle

    world = 2
    out = str(tmp_path / "gathered.pkl")
    store = str(tmp_path / "rendezvous")
    mp.start_processes(_rank_main, args=(world, store, out), nprocs=world, start_method="spawn", join=True)
    with open(out, "rb") as f:
        gathered = pickle.load(f)
    owners = [np.array(o) for _, o, _, _ in gathered]
    assert all(np.array_equal(owners[0], o) for o in owners)
    solved = {}
    for rank, owner, load, mine in gathered:
        for k, dist, r in mine:
            assert owner[k] == rank and k not in solved
            solved[k] = (dist, r)
    assert sorted(solved) == list(range(NGRAPHS))
    specs = dpg.rmat_batch_specs(NGRAPHS, seed=SEED, vmin=64, vmax=4096)
    for k in (0, 7, NGRAPHS - 1):
        _, dist, r = _solve(dpg, oracle, specs[k], k)
        assert np.array_equal(dist, solved[k][0])
        assert np.array_equal(r, solved[k][1])
