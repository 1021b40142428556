"""The replica path of bench.py on CPU: two gloo ranks on 127.0.0.1 reduce the
per-rank step time (max) and converged subsets (sum) as the GPU ranks do over
NCCL, and the reference arm's non-zero ranks exit without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        ms, n = bench.reduce_over_ranks(dist, 1.0 + rank, 100 + 10 * rank, "cpu")
        out.put((rank, ms, n))
    finally:
        dist.destroy_process_group()


def test_replicas_reduce_max_time_and_total_subsets():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.0, 210.0), (1, 2.0, 210.0)]


def test_reference_arm_other_ranks_exit_without_work():
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    args = argparse.Namespace(workload="hole1024", steps=1, warmup=1)
    assert bench.run_reference(args, 2, 1) == 0
