"""Multi-process host logic of bench.py --gpus N, on CPU with gloo.

One problem does not shard (every Omega block of one J couples every half step), so for the
single-J workloads N GPUs run N independent replicas; the only cross-rank steps are the
barrier and the max over ranks of the timed region.  The batched partial waves J = 0..40 are
independent of each other, so N GPUs split them, balanced by Omega-block count, step with no
exchange, and rank 0 gathers P(E) per J afterwards.  Two gloo ranks check the slowest-rank
time, the whole-job throughput, the partition and the gather.
"""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 + 25.0 * rank   # rank 1 is the slow one
        ms = bench.max_over_ranks(local_ms)
        value = bench.replica_throughput(local_ms, steps=40, blocks_per_replica=3)
        dist.barrier()
        out.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in res:
        assert ms == pytest.approx(125.0)
        assert value == pytest.approx(2 * 40 * 3 / 0.125)


def test_partial_waves_partition_balances_blocks():
    sys.path.insert(0, str(ROOT))
    import bench

    nb = [min(J, 20) + 1 for J in range(41)]          # the batched J = 0..40 run: 651 blocks
    for world in (1, 2, 3, 4, 8):
        parts = bench.partition_partial_waves(nb, world)
        assert sorted(j for p in parts for j in p) == list(range(41))   # every J exactly once
        loads = [sum(nb[j] for j in p) for p in parts]
        assert sum(loads) == 651
        assert max(loads) - min(loads) <= max(nb)       # within one partial wave of balance
    assert bench.partition_partial_waves([3, 1], 4)[2:] == [[], []]


def _gather_main(rank, world, port, out):
    import numpy as np
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        nb = [min(J, 20) + 1 for J in range(41)]
        mine = bench.partition_partial_waves(nb, world)[rank]
        got = bench.gather_crp({J: np.full(3, float(J)) for J in mine})
        dist.barrier()
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gather_p_of_e_per_partial_wave():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gather_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for rank, got in sorted(q.get(timeout=10) for _ in range(2)):
        assert sorted(got) == list(range(41))
        assert all(v == [float(J)] * 3 for J, v in got.items())
