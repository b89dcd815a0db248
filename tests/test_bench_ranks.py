"""The replica aggregation of bench.py on two gloo ranks (CPU): every rank
gets the slowest rank's time, and the whole-job rate counts every rank's
keys over it."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_setup()
        ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
        slowest = bench.max_over_ranks(ms, dist)
        rate = bench.whole_job_rate(1000, w, slowest / 1e3)
        out.put((r, local, w, slowest, rate))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_to_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, (r, local, w, slowest, rate) in enumerate(got):
        assert (r, local, w) == (rank, rank, 2)
        assert slowest == 15.0
        assert rate == pytest.approx(2 * 1000 / 0.015)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(100, 1, 0.5) == 200
