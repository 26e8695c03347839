"""Multi-process host logic of the replica benchmark (bench.py --gpus N), on CPU with gloo.

The propagator does not shard (every Omega block of one J couples every half step), so N GPUs
run N independent replicas; the only cross-rank steps are the barrier and the max over ranks
of the timed region.  Two gloo ranks check that both see the slowest rank's time and the
whole-job throughput N * steps * blocks / max(ms).
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
