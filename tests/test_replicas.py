"""The N-GPU path of bench.py is replicas only (solves are independent, no data-path
collective): each rank runs its own workload, and the harness needs a barrier and the
max-over-ranks of the timed milliseconds.  Checked here with two gloo ranks on CPU."""

import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.Dist()
    d.barrier()
    ms = 10.0 * (rank + 1)          # per-rank timed milliseconds
    worst = d.max(ms)
    d.barrier()
    q.put((rank, d.world, worst))
    d.close()


def test_two_rank_barrier_and_max_over_ranks():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 2, 20.0), (1, 2, 20.0)]
