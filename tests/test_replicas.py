"""Multi-process host logic of the replicas-only multi-GPU mode, on CPU with gloo (world size 2):
the slowest rank's time is what every rank reports, the job rate is world x per-replica work
over that time, and the reference arm prints from rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(100.0 + 50.0 * rank, dist, "cpu")
        rate = bench.whole_job_rate(world, 1e6 * 512, ms)
        buf = io.StringIO()
        with redirect_stdout(buf):
            if rank != 0:
                bench.run_reference(None)     # ranks other than 0 return without work
        q.put((rank, ms, rate, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_rank_timing_and_rate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate, out in res:
        assert ms == 150.0                         # max over ranks
        assert rate == pytest.approx(2 * 1e6 * 512 / 0.150)
        assert out == ""


def test_single_process_passthrough():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.whole_job_rate(1, 1000.0, 1000.0) == pytest.approx(1000.0)
