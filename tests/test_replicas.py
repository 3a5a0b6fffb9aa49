"""The N > 1 host logic of bench.py (one replica per rank, no collective on
the data path): max-over-ranks timing, whole-job sums and per-rank seeds, run
as two gloo ranks on the CPU."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        slowest = bench.allreduce_max(1.0 + rank, world)
        total = bench.allreduce_sum(10.0 * (rank + 1), world)
        case = bench.make_case(32, rank)
        # The seeded theta noise of the lowest level (below 200 m).
        out.put((rank, slowest, total, float(case.fields["th"][0, 0, 0])))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, max0, sum0, th0), (r1, max1, sum1, th1) = res
    assert (r0, r1) == (0, 1)
    # Every rank sees the slowest rank's time and the whole-job sum.
    assert max0 == max1 == 2.0
    assert sum0 == sum1 == 30.0
    # Each replica has its own seed.
    assert th0 != th1


def test_single_rank_helpers_are_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.allreduce_max(3.5, 1) == 3.5
    assert bench.allreduce_sum(3.5, 1) == 3.5
    bench.barrier(1)
