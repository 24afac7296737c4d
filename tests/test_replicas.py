"""Multi-rank plumbing on CPU ranks (gloo, world size 2): the timing maximum
over ranks, the barrier, and a deterministic style sharding that covers
every job exactly once."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from vkhr_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, size, port, costs, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(size),
                      LOCAL_RANK=str(rank))
    replicas.init("gloo")
    replicas.barrier()
    m = replicas.max_over_ranks(10.0 * (rank + 1))
    mine = replicas.shard(costs, rank, size)
    out.put((rank, m, mine))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks():
    costs = [5.0, 136.0, 40.0, 7.0, 90.0, 12.0, 64.0, 33.0, 8.0, 120.0, 6.0, 18.0, 77.0, 25.0, 9.0, 50.0]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort()
    assert all(m == 20.0 for _, m, _ in results)
    a, b = results[0][2], results[1][2]
    assert sorted(a + b) == list(range(len(costs))) and not set(a) & set(b)
    la, lb = sum(costs[i] for i in a), sum(costs[i] for i in b)
    assert abs(la - lb) <= max(costs)  # balanced within one job


def test_single_process_defaults():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.shard([1.0, 2.0, 3.0], 0, 1) == [0, 1, 2]
