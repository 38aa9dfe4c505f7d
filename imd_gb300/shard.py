"""Sharding of independent cells over ranks (one process per GPU).

Batched relaxations shard by cell: every rank relaxes its own cells and no
data moves between ranks while they run.  At the end rank 0 gathers the
per-cell results in the original cell order.  Host logic only; the
collectives are torch.distributed's, on whatever backend the process group
has (gloo in the CPU tests).
"""
from __future__ import annotations

import numpy as np


def shard_cells(sizes, world: int) -> list:
    """Split cells into `world` shards of nearly equal atom count.

    sizes: atoms per cell.  Cells are taken largest first and each goes to
    the shard with the fewest atoms so far (ties: the lower rank), so the
    slowest rank, which sets the batch's time, holds as few atoms as this
    greedy rule allows.  Returns one sorted index array per rank."""
    sizes = np.asarray(sizes, np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    load = np.zeros(world, np.int64)
    out = [[] for _ in range(world)]
    for c in np.argsort(-sizes, kind="stable"):
        r = int(np.argmin(load))
        out[r].append(int(c))
        load[r] += sizes[c]
    return [np.array(sorted(o), np.int64) for o in out]


def gather_cell_results(local: dict, index, ncells: int, dist=None):
    """Assemble per-cell result arrays from every rank on rank 0.

    local: name -> array over this rank's cells (in the order of `index`);
    index: the global cell numbers of this rank's cells.  Returns the
    assembled dict on rank 0 (None elsewhere); without a process group the
    local arrays are simply placed."""
    index = np.asarray(index, np.int64)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        parts = [(index, local)]
    else:
        world = dist.get_world_size()
        obj = [None] * world if dist.get_rank() == 0 else None
        dist.gather_object((index, local), obj, dst=0)
        if dist.get_rank() != 0:
            return None
        parts = obj
    out = {}
    seen = np.zeros(ncells, bool)
    for idx, arrs in parts:
        if np.any(seen[idx]):
            raise ValueError("a cell was relaxed on two ranks")
        seen[idx] = True
        for k, v in arrs.items():
            v = np.asarray(v)
            if k not in out:
                out[k] = np.zeros((ncells,) + v.shape[1:], v.dtype)
            out[k][idx] = v
    if not seen.all():
        raise ValueError("cells missing from the gathered results: %s"
                         % np.flatnonzero(~seen)[:10].tolist())
    return out


def max_over_ranks(x: float, dist=None) -> float:
    """The largest value over all ranks (the batch's time is its slowest
    rank's)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])
