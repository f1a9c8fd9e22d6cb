"""The multi-rank path of bench.py on CPU (gloo, world size 2): the path runs
independent replicas, one per GPU, and the only exchange is the timing, the
slowest rank's time, from which the whole-job rate follows; the reference arm
runs on rank 0 alone."""
import argparse
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as td
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, "cpu")   # rank r took 10 + 5 r seconds
        q.put((rank, slowest, bench.job_rate(world, 100, slowest)))
    finally:
        td.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(2):
        rank, slowest, rate = q.get(timeout=120)
        got[rank] = (slowest, rate)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's 15 s; 2 replicas x 100 steps in 15 s
    assert got == {0: (15.0, 200.0 / 15.0), 1: (15.0, 200.0 / 15.0)}


def test_reference_arm_other_ranks_do_no_work():
    sys.path.insert(0, ROOT)
    import bench
    args = argparse.Namespace(warmup=1, steps=1)
    assert bench.run_reference(args, rank=1, world=2) == 0
