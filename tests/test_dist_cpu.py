"""The multi-process bench path on CPU: two gloo ranks shard a batch of independent blocks (longest first, like the
reference's claim_block, src/core/blocks.c:148-178) with no data-path collective, then agree on the max step time."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, sizes, q):
    import torch.distributed as dist

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    w, r, lr = bench.dist_env()
    assert (w, r, lr) == (world, rank, rank)
    bench.dist_init(world, "gloo")
    mine = bench.shard(sizes, rank, world)
    work = float(sum(sizes[i] for i in mine))
    bench.barrier(world)
    m = bench.reduce_max(work, world)
    q.put((rank, mine, work, m))
    dist.destroy_process_group()


def test_two_rank_sharding_and_max_reduction():
    sizes = [5, 100, 7, 64, 64, 1, 33, 90, 2, 50]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    all_blocks = sorted(out[0][1] + out[1][1])
    assert all_blocks == list(range(len(sizes)))          # every block exactly once
    assert not set(out[0][1]) & set(out[1][1])
    loads = [o[2] for o in out]
    assert abs(loads[0] - loads[1]) <= max(sizes)          # longest-first keeps ranks balanced
    assert out[0][3] == out[1][3] == max(loads)            # both ranks see the max


@pytest.mark.parametrize("world", [1, 3, 4])
def test_shard_partitions(world):
    sizes = list(range(1, 40))
    parts = [bench.shard(sizes, r, world) for r in range(world)]
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(sizes)))
