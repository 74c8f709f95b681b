"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): the process group comes up from the
torchrun environment variables, the barrier releases both ranks, the timed region's duration is the max over
ranks, the whole-job value counts every rank's replica, and the reference arm does its work on rank 0 only."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    try:
        import torch.distributed as dist

        import bench

        r, local, w = bench.dist_init()
        assert (r, local, w) == (rank, rank, world)
        assert dist.get_backend() == "gloo"
        bench.barrier(w)
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, w)  # each rank's timed-region duration
        rays_per_step, steps = 1000, 4
        value = w * rays_per_step * steps / (ms / 1e3)
        # the reference arm returns at once on ranks other than 0 (rank 0 alone runs and prints it)
        returned = None
        if rank != 0:

            class Args:
                warmup, steps = 1, 1

            returned = bench.run_reference(Args(), rank, w)
        bench.barrier(w)
        dist.destroy_process_group()
        q.put((rank, ms, value, returned))
    except Exception as e:  # noqa: BLE001 - report to the parent
        q.put((rank, "error", repr(e), None))


@pytest.mark.timeout(120)
def test_two_rank_gloo_timing_and_aggregation():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=100) for _ in procs]
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    out.sort()
    for rank, ms, value, returned in out:
        assert ms != "error", value
        assert ms == 15.0  # the max over ranks, seen by both
        assert value == pytest.approx(2 * 1000 * 4 / 0.015)
        assert returned is None
