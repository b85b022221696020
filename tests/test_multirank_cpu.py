"""The replicas path of bench.py with two ranks on CPU (gloo): setup, barrier, max over ranks of
the step time and the whole-job rate, as the GPU run does them over NCCL."""
import os
import socket
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank), RAL_DIST_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    import torch.distributed as dist
    args = argparse.Namespace(impl="ours")
    w, r, local = bench.dist_setup(args)
    bench.barrier(w)
    ms = bench.max_over_ranks(w, 10.0 + 5.0 * r)       # rank 1 is the slow one
    rate = bench.job_rate(w, 1_000_000, ms)
    out.put((r, w, local, ms, rate))
    dist.destroy_process_group()


def test_two_replicas_agree_on_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == 15.0 for r in res)                      # max over ranks
    assert all(abs(r[4] - 2 * 1_000_000 / 0.015) < 1e-3 for r in res)   # both ranks' rows / slowest time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    w, r, local = bench.dist_setup(argparse.Namespace(impl="ours"))
    assert (w, r, local) == (1, 0, 0)
    assert bench.max_over_ranks(1, 3.0) == 3.0
    assert bench.job_rate(1, 500, 1000.0) == 500.0
