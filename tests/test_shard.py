"""Batched worlds sharded over ranks: the multi-GPU path of the batch
benchmark, exercised as two gloo ranks on the CPU.

Each rank takes its contiguous range of worlds from `shard.partition`,
steps only those worlds (here through the CPU oracle, which has the same C
API as the GPU library), and the ranks gather their per-world results.  The
gathered results must equal one process stepping every world, and every
world must be stepped by exactly one rank.
"""
import os
import random
import socket
import sys

import numpy as np
import pytest

from chipmunk2d_gb300.shard import partition, rank_range

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SIZES = [8, 40, 9, 120, 16, 70, 12, 33, 8, 64, 21, 15]
STEPS = 20


def test_partition_tiles_and_balances():
    rng = random.Random(7)
    for _ in range(500):
        n = rng.randint(0, 80)
        r = rng.randint(1, 8)
        costs = [rng.randint(0, 512) for _ in range(n)]
        parts = partition(costs, r)
        assert len(parts) == r and parts[0][0] == 0 and parts[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
        if n >= r:
            assert all(hi > lo for lo, hi in parts)
        if n >= 2 * r and n:
            share = sum(costs) / r
            assert max(sum(costs[lo:hi]) for lo, hi in parts) <= share + max(costs)
    assert partition([5, 5, 5, 5], 2) == [(0, 2), (2, 4)]
    assert rank_range([1, 1, 1, 9], 1, 2) == (3, 4)
    with pytest.raises(ValueError):
        partition([1], 0)


def _step_worlds(lib, indices):
    from chipmunk2d_gb300 import Scene
    out = {}
    for i in indices:
        sc = Scene(lib, 4, SIZES[i], seed=1000 + i)
        sc.step(1 / 60, STEPS)
        out[i] = sc.bodies()
        sc.free()
    return out


def _rank_main(rank, world, port, oracle_so, result_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    from chipmunk2d_gb300 import bind
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = rank_range(SIZES, rank, world)
        mine = _step_worlds(bind(oracle_so), range(lo, hi))
        gathered = [None] * world
        dist.all_gather_object(gathered, {"range": (lo, hi), "bodies": mine})
        dist.barrier()
        if rank == 0:
            np.save(result_path, np.array(gathered, dtype=object), allow_pickle=True)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_equal_one_process(oracle_lib, tmp_path):
    import torch.multiprocessing as mp
    from conftest import ORACLE_SO
    result_path = str(tmp_path / "gathered.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), ORACLE_SO, result_path), nprocs=2,
                       join=True, start_method="spawn")
    gathered = list(np.load(result_path, allow_pickle=True))
    ranges = [g["range"] for g in gathered]
    assert ranges == partition(SIZES, 2)
    stepped = sorted(i for g in gathered for i in g["bodies"])
    assert stepped == list(range(len(SIZES)))          # every world, once
    serial = _step_worlds(oracle_lib, range(len(SIZES)))
    for g in gathered:
        for i, b in g["bodies"].items():
            np.testing.assert_array_equal(b, serial[i])
