"""Multi-GPU replica logic on CPU: two gloo ranks partition the images and agree on the job time.

The path has no data-path collective (independent searches per image), so this covers the host side of N > 1: the
partition each rank computes on its own, and the max-over-ranks reduction of the timed region."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, sizes, out):
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "rust-compress_gb300"))
    import torch.distributed as dist

    from rcg import replicas

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert replicas.env_rank() == (rank, world, rank)
    mine = replicas.shard(sizes, rank, world)
    work = float(sum(sizes[i] for i in mine))
    out[rank] = (mine, replicas.max_over_ranks(work, dist), replicas.sum_over_ranks(len(mine), dist))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_ranks_partition_the_images_and_agree_on_the_max(world):
    import rcg.synth as synth

    sizes = [w * h for w, h in synth.log_uniform_sizes(2, 64)]
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, sizes, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    shards = [out[r][0] for r in range(world)]
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(sizes)))  # every image exactly once
    loads = [sum(sizes[i] for i in s) for s in shards]
    assert all(out[r][1] == max(loads) for r in range(world))  # every rank sees the slowest rank's load
    assert all(out[r][2] == len(sizes) for r in range(world))
    assert max(loads) <= 1.25 * sum(loads) / world + max(sizes)  # balanced


def test_single_process_shard_is_everything():
    import rcg.replicas as replicas

    assert replicas.shard([5, 1, 3], 0, 1) == [0, 1, 2]
    assert replicas.max_over_ranks(3.5) == 3.5
