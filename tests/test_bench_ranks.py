"""CPU tests of the multi-process side of bench.py (world size 2 over gloo): every rank runs its own replica and the
job's time is the slowest rank's; the reference arm runs on rank 0 only."""

import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch.multiprocessing as mp

from tests.conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world_2():
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    assert out[0] == 2.5 and out[1] == 2.5


def test_max_over_ranks_without_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25


def test_reference_arm_prints_on_rank_zero_only():
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_arm(argparse.Namespace(steps=1, warmup=1), rank=1, world=2)
    assert buf.getvalue() == ""
