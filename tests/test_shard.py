"""Sharding of independent cells over ranks, on CPU: two gloo ranks split a
batch of cells by atom count, produce per-cell results, and rank 0 gathers
them back in the original cell order; the batch time is the slowest rank's.
No GPU: the relaxation is replaced by a deterministic function of the cell."""
import os
import socket

import numpy as np
import pytest

from imd_gb300 import shard


def test_shard_cells_balances_and_covers():
    rng = np.random.default_rng(0)
    sizes = np.exp(rng.uniform(np.log(500), np.log(20000), 512)).astype(int)
    for world in (1, 2, 3, 8):
        parts = shard.shard_cells(sizes, world)
        allc = np.sort(np.concatenate(parts))
        assert np.array_equal(allc, np.arange(len(sizes)))
        loads = np.array([sizes[p].sum() for p in parts])
        # greedy largest-first: no shard exceeds the mean by more than the largest cell
        assert loads.max() - loads.mean() <= sizes.max()
    with pytest.raises(ValueError):
        shard.shard_cells(sizes, 0)


def test_gather_without_process_group():
    out = shard.gather_cell_results({"e": np.array([3.0, 1.0])}, [1, 0], 2)
    assert np.array_equal(out["e"], [1.0, 3.0])
    with pytest.raises(ValueError):
        shard.gather_cell_results({"e": np.array([3.0])}, [1], 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, sizes, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard.shard_cells(sizes, world)[rank]
        local = {"epot": -3.5 * sizes[mine].astype(float), "nfc": (sizes[mine] % 97).astype(np.int32),
                 "rank": np.full(len(mine), rank, np.int32)}
        t = float(sizes[mine].sum())           # stands in for the rank's wall time
        tmax = shard.max_over_ranks(t, dist)
        out = shard.gather_cell_results(local, mine, len(sizes), dist)
        if rank == 0:
            q.put((out, tmax))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_in_order():
    import torch.multiprocessing as mp
    rng = np.random.default_rng(1)
    sizes = np.exp(rng.uniform(np.log(500), np.log(20000), 64)).astype(np.int64)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    out, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert np.allclose(out["epot"], -3.5 * sizes)
    assert np.array_equal(out["nfc"], sizes % 97)
    assert set(np.unique(out["rank"])) == {0, 1}
    parts = shard.shard_cells(sizes, 2)
    assert tmax == max(float(sizes[p].sum()) for p in parts)
