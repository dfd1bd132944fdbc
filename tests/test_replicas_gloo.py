"""The N-process path of bench.py, run as two gloo ranks on the CPU: the solve
does not shard (one particle's FFTs would need an all-to-all transpose), so
N GPUs run N replicas and the job's time is the slowest rank's, reduced over
the process group exactly as bench.py does with NCCL."""
import os
import socket
import sys

import pytest

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
        out[rank] = bench._max_over_ranks(10.0 + 2.5 * rank, dist, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_slowest_replica_time_reaches_every_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 12.5, 1: 12.5}


def test_single_process_keeps_its_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench._max_over_ranks(7.25, None, "cpu") == 7.25
