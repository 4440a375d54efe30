"""Sharding a sweep over processes (one per GPU): the partition and the merge, on the CPU.

gopf_sweep_partition is host code of the library (no device needed).  The
world-size-2 test runs two gloo ranks: each steps the instances it owns with
the FP64 oracle (small grids, so it runs in seconds), the per-instance results
are all-gathered and merged, and the merged list must equal a single-process
run instance for instance.  The GPU path (bench.py --workload sweep under
torchrun) uses the same partition and merge, with a device batch as the work.
"""
import os
import socket

import numpy as np
import pytest

SIDES = [128, 256, 384, 512, 768, 1024]


def sweep_sides(n=64, seed=2):
    from gopf_gb300.synthetic import splitmix64_uniform

    u = splitmix64_uniform(seed, 3 * n)
    return [SIDES[min(int(u[3 * i] * 6), 5)] for i in range(n)]


def test_partition_is_deterministic_and_complete():
    from gopf_gb300 import sweep

    cells = [s * s for s in sweep_sides()]
    for world in (1, 2, 3, 4, 8):
        owner, load = sweep.partition(cells, world)
        assert owner == sweep.partition(cells, world)[0]
        assert len(owner) == len(cells) and all(0 <= r < world for r in owner)
        assert sum(load) == sum(cells)
        for r in range(world):
            assert load[r] == sum(c for c, o in zip(cells, owner) if o == r)
        # greedy longest-first packing: no rank exceeds the mean by more than the largest instance
        assert max(load) <= sum(cells) / world + max(cells)
        # every instance is owned by exactly one rank
        got = sorted(i for r in range(world) for i in sweep.owned(cells, r, world))
        assert got == list(range(len(cells)))


def test_partition_ties_and_edges():
    from gopf_gb300 import sweep

    owner, load = sweep.partition([10, 10, 10, 10], 2)
    assert owner == [0, 1, 0, 1] and load == [20, 20]
    owner, load = sweep.partition([], 3)
    assert owner == [] and load == [0, 0, 0]
    owner, load = sweep.partition([5, 1], 4)  # more ranks than instances: the extra ranks own nothing
    assert owner == [0, 1] and load == [5, 1, 0, 0]
    with pytest.raises(ValueError):
        sweep.partition([1, -2], 2)
    with pytest.raises(ValueError):
        sweep.partition([1, 2], 0)


def test_merge_rejects_duplicates_and_gaps():
    from gopf_gb300 import sweep

    assert sweep.merge([{0: "a", 2: "c"}, {1: "b"}], 3) == ["a", "b", "c"]
    with pytest.raises(ValueError):
        sweep.merge([{0: 1}, {0: 1, 1: 2}], 2)
    with pytest.raises(ValueError):
        sweep.merge([{0: 1}], 2)


# ---- two gloo ranks ----

def _oracle_work(params):
    """Step each owned instance (side, gamma, M) 5 Euler steps with the oracle; the result is the
    field's checksum pair (sum, sum of squares)."""
    from gopf_gb300.synthetic import uniform_field
    from oracle import oracle as O

    def work(indices):
        out = {}
        for i in indices:
            side, gamma, M = params[i]
            o = O.cahn_hilliard([side, side], gamma=gamma, M=M)
            o.set_field(0, uniform_field(1000 + i, side * side, 0.5, 0.05))
            o.step_euler(0.05, 5)
            f = o.field(0).real
            out[i] = (float(f.sum()), float((f * f).sum()))
        return out

    return work


def _small_params():
    from gopf_gb300.synthetic import splitmix64_uniform

    u = splitmix64_uniform(2, 3 * 16)
    small = [8, 16, 24, 32, 48, 64]
    return [(small[min(int(u[3 * i] * 6), 5)], 0.2 + 1.8 * u[3 * i + 1], 0.5 + 1.5 * u[3 * i + 2]) for i in range(16)]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    from gopf_gb300 import sweep

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        params = _small_params()
        cells = [p[0] ** 2 for p in params]
        res = sweep.run_sharded(cells, _oracle_work(params), rank, world)
        q.put((rank, sweep.owned(cells, rank, world), res))
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_gloo_ranks_merge_equals_single_process():
    import torch.multiprocessing as mp

    from gopf_gb300 import sweep

    params = _small_params()
    cells = [p[0] ** 2 for p in params]
    single = sweep.run_sharded(cells, _oracle_work(params), 0, 1)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    owners = {}
    for rank, mine, res in got:
        assert res == single  # every rank holds the merged result, equal to one process's
        for i in mine:
            assert i not in owners
            owners[i] = rank
    assert sorted(owners) == list(range(len(params)))
    assert set(owners.values()) == {0, 1}  # both ranks did work
