"""The N>1 (replicas) path on CPU: world_size 2 over gloo. Each rank times its
own work; the job's time is the slowest rank's and the throughput counts every
rank's units."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from hashinator_gb300 import dist as hd
    dist.barrier()
    elapsed = 0.5 + rank  # rank 1 is the slow one
    thr, t = hd.aggregate_throughput(1000, elapsed)
    seeds = [None] * world
    dist.all_gather_object(seeds, hd.replica_seed(11, rank))
    q.put((rank, thr, t, seeds))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, thr, t, seeds in res:
        assert t == pytest.approx(1.5)                # max over ranks
        assert thr == pytest.approx(2 * 1000 / 1.5)   # all ranks' units / slowest time
        assert len(set(seeds)) == 2                   # replicas use distinct inputs


def test_single_process_identity():
    from hashinator_gb300 import dist as hd
    assert hd.max_over_ranks(3.0) == 3.0
    assert hd.aggregate_throughput(10, 2.0) == (5.0, 2.0)
