"""The bench's multi-rank host logic on CPU ranks (gloo, world size 2, 127.0.0.1): the whole-job value is the slowest
rank's rate times the ranks, and the barrier bracket returns on every rank. The GPU ranks use the same functions
over NCCL."""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, values, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench

    bench.bracket(dist)
    out[rank] = bench.whole_job(values[rank], world, dist)
    bench.bracket(dist)
    dist.destroy_process_group()


def test_whole_job_is_slowest_rank_times_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context('spawn')
    with ctx.Manager() as m:
        out = m.dict()
        values = [120.0, 80.0]
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, values, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        assert dict(out) == {0: 160.0, 1: 160.0}


def test_whole_job_single_rank():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.whole_job(42.5, 1) == 42.5
