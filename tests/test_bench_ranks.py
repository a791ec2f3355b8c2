"""The multi-rank path of bench.py (one replica per GPU, the job's time is the slowest rank's),
exercised with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

import importlib.util

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = _bench()
    t = b.max_over_ranks(1.0 + rank, dist, "cpu")   # rank 1 is the slower one
    out[rank] = (t, b.job_value(world, 1000, 2, t))
    dist.destroy_process_group()


def test_two_ranks_report_the_slowest_and_the_whole_job():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        t, v = res[r]
        assert t == 2.0
        assert v == world * 1000 * 2 / 2.0


def test_single_rank_is_unchanged():
    b = _bench()
    assert b.max_over_ranks(3.5, None, "cpu") == 3.5
    assert b.job_value(1, 100, 3, 2.0) == 150.0
