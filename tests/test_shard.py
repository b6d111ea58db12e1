"""Sharding of ensembles across ranks (resaxs_gb300/shard.py): the partition
and the one all-reduce that combines the ranks, run as world_size-2 gloo
ranks on the CPU (the per-member curves are stand-ins; the GPU pass each rank
runs is covered by tests/test_batch_gpu.py)."""
import os
import socket

import numpy as np
import pytest

from resaxs_gb300 import shard


def test_partition_covers_every_member_once():
    rng = np.random.default_rng(0)
    sizes = rng.integers(1000, 30001, 256)
    for world in (1, 2, 3, 4, 8):
        parts = shard.partition_members(sizes, world)
        assert len(parts) == world
        flat = sorted(m for p in parts for m in p)
        assert flat == list(range(len(sizes)))
        loads = shard.partition_loads(sizes, parts)
        biggest = max(int(n) * (int(n) - 1) // 2 for n in sizes)
        # LPT: no rank exceeds the mean by more than one member's work
        assert max(loads) - sum(loads) / world <= biggest


def test_partition_is_deterministic_and_handles_edges():
    sizes = [5, 5, 5, 100, 2]
    assert shard.partition_members(sizes, 2) == shard.partition_members(list(sizes), 2)
    assert shard.partition_members([], 3) == [[], [], []]
    parts = shard.partition_members([10, 20], 4)
    assert sorted(m for p in parts for m in p) == [0, 1]
    with pytest.raises(ValueError):
        shard.partition_members([1], 0)


def test_ensemble_average_without_process_group():
    s = np.array([2.0, 4.0, 6.0])
    np.testing.assert_allclose(shard.ensemble_average(s, 2), [1.0, 2.0, 3.0])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, sizes, curves, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        parts = shard.partition_members(sizes, world)
        mine = parts[rank]
        local = curves[mine].sum(axis=0) if mine else np.zeros(curves.shape[1])
        avg = shard.ensemble_average(local, len(mine))
        np.save(os.path.join(out_dir, f"avg{rank}.npy"), avg)
        np.save(os.path.join(out_dir, f"mine{rank}.npy"), np.array(mine, np.int64))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_to_the_full_average(tmp_path):
    import torch.multiprocessing as mp
    rng = np.random.default_rng(1)
    sizes = rng.integers(300, 3000, 37)
    curves = rng.normal(size=(37, 51)) * 1e6
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), sizes, curves, str(tmp_path)),
                       nprocs=world, join=True, start_method="spawn")
    full = curves.mean(axis=0)
    seen = []
    for r in range(world):
        np.testing.assert_allclose(np.load(tmp_path / f"avg{r}.npy"), full, rtol=1e-12)
        seen += np.load(tmp_path / f"mine{r}.npy").tolist()
    assert sorted(seen) == list(range(37))
