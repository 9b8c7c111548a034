"""Multi-GPU in this path is replicas only: every rank applies its own operator and the harness reports all ranks' DoF
over the slowest rank's time.  The rank-side logic (max over ranks, whole-job rate) runs here as two gloo processes
on the CPU, as it would over NCCL with one rank per GPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # Rank r was slowest in the first timing, fastest in the second.
        res = bench.max_over_ranks([10.0 + rank, 20.0 - rank, 3.0], world)
        out[rank] = res
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_rate_with_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        assert out[r] == [11.0, 20.0, 3.0]
    import sys

    sys.path.insert(0, ROOT)
    import bench

    # 2 replicas x 16,974,593 DoF x 100 steps over the slowest rank's 700 ms.
    assert bench.replica_rate(16974593, 2, 100, 700.0) == pytest.approx(2 * 16974593 * 100 / 0.7 / 1e9)
