"""The multi-rank host logic with world_size 2 on gloo (CPU): throughput
aggregation as bench.py reports it under torchrun, and the incumbent
exchange between replicas."""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from wsbb_gb300 import replicas as R
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r bounded 1000 * (r + 1) nodes in 2 + r seconds
        total, slow, rate = R.aggregate(1000 * (rank + 1), 2.0 + rank)
        # incumbents: rank 1 holds the better one; then a tie at 50
        perm = np.arange(6, dtype=np.int32)[::-1] if rank == 1 else np.arange(6, dtype=np.int32)
        c1, p1, o1 = R.min_incumbent(100 - 10 * rank, perm)
        c2, p2, o2 = R.min_incumbent(50, perm)
        out.put((rank, total, slow, rate, c1, p1.tolist(), o1, c2, p2.tolist(), o2,
                 R.replica_seed(rank)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_aggregate_and_exchange_incumbents():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total, slow, rate, c1, p1, o1, c2, p2, o2, seed in res:
        assert total == 3000 and slow == 3.0 and rate == pytest.approx(1000.0)
        assert (c1, o1) == (90, 1) and p1 == [5, 4, 3, 2, 1, 0]
        assert (c2, o2) == (50, 0) and p2 == [0, 1, 2, 3, 4, 5]
        assert seed == rank


def test_single_process_falls_back_to_local_values():
    from wsbb_gb300 import replicas as R
    assert R.aggregate(10, 2.0) == (10.0, 2.0, 5.0)
    c, p, o = R.min_incumbent(7, [2, 0, 1])
    assert (c, o) == (7, 0) and p.tolist() == [2, 0, 1]
