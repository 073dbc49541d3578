"""bench.py's replica aggregation (N > 1): every rank times its own copy of
the workload, the job time is the slowest rank's, the value the sum over
ranks.  Two gloo processes on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(2.0 + rank, world)   # rank 1 is slower
    out.put((rank, ms, bench.replica_value(ms, world)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
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
    assert [r[1] for r in res] == [3.0, 3.0]
    assert res[0][2] == pytest.approx(2 * 1e3 / 3.0)


def test_single_rank_is_unchanged():
    import bench
    assert bench.max_over_ranks(4.5, 1) == 4.5
    assert bench.replica_value(4.0, 1) == 250.0
