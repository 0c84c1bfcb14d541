"""Host logic of bench.py's N>1 replica runs, on CPU with the gloo backend:
the job time is the maximum over ranks (every replica does the same work,
the slowest sets the time), and the reference arm runs on rank 0 only."""
import argparse
import io
import os
import sys
from contextlib import redirect_stdout

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _worker(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    try:
        assert bench.dist_env() == (world, rank, rank)
        out.put((rank, bench.max_over_ranks(times[rank], dist)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [12.5, 31.25]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 31.25, 1: 31.25}


def test_max_over_ranks_without_group_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(p=4, nx=64, steps=2, warmup=3)
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(args) == 0
    assert buf.getvalue() == ""  # no line and no work on the other ranks
