"""Multi-rank bench logic on CPU (gloo, world size 2): the path shards as independent replicas,
and the only collective is the max of the timed region over ranks."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        ms = [120.0, 80.0][rank]  # rank 0 is the slower replica
        out[rank] = bench.job_rate(ms, 1000, 10, world)
        # the reference arm: rank 0 alone works; the others return without output
        if rank == 1:
            bench.reference_arm(None, rank, world)
    finally:
        torch.distributed.destroy_process_group()


def test_job_rate_is_bounded_by_the_slowest_rank():
    world, port = 2, _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    for rank in range(world):
        ms_max, value = out[rank]
        assert ms_max == 120.0
        assert value == pytest.approx(world * 1000 * 10 / 0.120)


def test_job_rate_single_rank():
    sys.path.insert(0, str(ROOT))
    import bench

    ms_max, value = bench.job_rate(50.0, 2000, 4, 1)
    assert ms_max == 50.0 and value == pytest.approx(2000 * 4 / 0.05)
