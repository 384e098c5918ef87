"""The replica path of bench.py on CPU: two gloo ranks, the timed region's
max over ranks and the whole-job rate (units of all ranks / that time)."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    worst = bench.max_over_ranks(torch, dist, torch.device("cpu"), ms)
    out[rank] = (worst, bench.whole_job_rate(1000.0, world, worst * 1e-3))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest():
    world, port = 2, _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (15.0, pytest.approx(2000.0 / 0.015))
