"""Replica sharding on two gloo ranks (CPU): blocks cover every entry once, results
gather in rank order, timing reduces to the maximum."""

import os
import socket

import pytest
import torch.multiprocessing as mp

from custom_madi_gb300.sharding import shard, shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 256, 1001):
        for world in (1, 2, 3, 8):
            blocks = [shard_range(n, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(blocks[i][1] == blocks[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from custom_madi_gb300.sharding import gather_to_rank0, max_over_ranks
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    entries = list(range(10))
    mine = shard(entries, rank, world)
    result = [e * e for e in mine]
    t = max_over_ranks(1.0 + rank)
    got = gather_to_rank0(result)
    if rank == 0:
        q.put((got, t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_shard_and_gather():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    mp.start_processes(_worker, args=(2, port, q), nprocs=2, join=True, start_method="spawn")
    got, t = q.get(timeout=60)
    assert [x for part in got for x in part] == [e * e for e in range(10)]
    assert t == 2.0
