"""Multi-GPU replica path on the host: two gloo ranks on CPU (no GPU needed).

The bench's N > 1 launch runs one rank per GPU, each with its own seeds and no
collective in the sweep; the whole-job time is the maximum over ranks.  This test
runs that reduction with world_size 2 over gloo and checks the seeds and the rate.
"""
import os
import socket

import torch.multiprocessing as mp

from alf_gb300 import replicas


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [1.0 + rank, 10.0 - rank]  # rank 1 is slower in the first entry
        out[rank] = replicas.max_over_ranks(local)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0] == out[1] == [2.0, 10.0]
    assert replicas.whole_job_rate(world, 3, 5, 2.0) == 15.0


def test_replica_seeds_are_distinct():
    seeds = {replicas.replica_seed(7, r, c) for r in range(8) for c in range(128)}
    assert len(seeds) == 8 * 128
