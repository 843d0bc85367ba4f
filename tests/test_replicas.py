"""The multi-GPU logic of bench.py on CPU: world_size 2 over gloo (127.0.0.1).

The time step does not shard (one coupled solve), so N GPUs run replicas;
the batched ensemble's cases are independent and are partitioned across
ranks with no data exchange.  What needs checking without GPUs: every rank
gets the slowest rank's time (the reported value uses it), and the case
partition covers every case exactly once with balanced cell counts."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, sizes, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.0 + 0.25 * rank, dist)
        mine = bench.shard_cases(sizes, rank, world)
        shards = [None] * world
        dist.all_gather_object(shards, mine)
        q.put((rank, t, shards))
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_and_case_partition():
    pytest.importorskip("torch")
    sizes = [32 * 48 * 64, 96 ** 3, 64 ** 3, 80 * 32 * 96, 48 ** 3, 96 * 64 * 32, 32 ** 3]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [t for _, t, _ in out] == [1.25, 1.25]
    shards = out[0][2]
    assert shards == out[1][2]
    cover = sorted(i for s in shards for i in s)
    assert cover == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(sizes)
