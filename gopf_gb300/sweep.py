"""Parameter sweeps sharded over processes, one per GPU.

gopf runs a sweep as one pf.Solver per parameter set, one after the other
(README.md:21-33).  The instances are independent, so several GPUs split them
with no exchange on the data path: every rank computes the same partition
(gopf_sweep_partition: greedy bin packing on cell counts, in the library),
steps its own instances as one batch (gopf_batch_*), and the per-instance
results are merged on the host.  The only collective is the final gather of
those results (torch.distributed object gather; gloo or NCCL).
"""
from __future__ import annotations

import ctypes
from typing import Callable, Sequence

import numpy as np

from . import _lib


def partition(cells: Sequence[int], world: int):
    """(owner, rank_cells): owner[i] is the rank that steps instance i; rank_cells[r] the cells of
    rank r.  Deterministic: every rank computes the same answer from the cell counts alone."""
    L = _lib.load()
    n = len(cells)
    c = np.ascontiguousarray(cells, dtype=np.int64)
    owner = np.empty(max(n, 1), dtype=np.int32)
    load = np.empty(world, dtype=np.int64)
    rc = L.gopf_sweep_partition(c.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), n, int(world),
                                owner.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                load.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
    if rc != 0:
        raise ValueError(f"gopf_sweep_partition: {_lib.STATUS.get(rc, rc)}")
    return owner[:n].tolist(), load.tolist()


def owned(cells: Sequence[int], rank: int, world: int) -> list[int]:
    """The instances rank `rank` steps, in increasing index order."""
    owner, _ = partition(cells, world)
    return [i for i, r in enumerate(owner) if r == rank]


def merge(parts: Sequence[dict], n: int) -> list:
    """Per-instance results of every rank -> one list in instance order.  Fails when an instance is
    missing or reported by two ranks."""
    out = [None] * n
    seen = set()
    for part in parts:
        for i, v in part.items():
            if not 0 <= i < n:
                raise ValueError(f"instance {i} is out of range")
            if i in seen:
                raise ValueError(f"instance {i} was reported by two ranks")
            seen.add(i)
            out[i] = v
    missing = [i for i in range(n) if i not in seen]
    if missing:
        raise ValueError(f"instances {missing} were reported by no rank")
    return out


def run_sharded(cells: Sequence[int], work: Callable[[list[int]], dict], rank: int = 0, world: int = 1,
                group=None) -> list:
    """Step this rank's share with `work(indices) -> {index: result}` and return every instance's
    result on every rank (an all-gather of the per-rank dicts when world > 1)."""
    mine = owned(cells, rank, world)
    res = work(mine)
    if set(res) != set(mine):
        raise ValueError("work() must return exactly the instances it was given")
    if world == 1:
        return merge([res], len(cells))
    import torch.distributed as dist

    parts = [None] * world
    dist.all_gather_object(parts, res, group=group)
    return merge(parts, len(cells))
