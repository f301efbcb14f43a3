"""bench.py --gpus N runs N independent replicas (the solve does not shard):
the rank plumbing -- process group, barrier, max over ranks, rank-0-only
reference arm -- on two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    r, w, local = bench.dist_setup(world)
    bench.barrier(w)
    m = bench.max_over_ranks(float(10 * (r + 1)), w)

    class Args:
        workload, gpus, steps, warmup = "square20k", world, 1, 0

    if r != 0:
        bench.run_reference(Args, r, w)  # returns at once on every rank but 0
    q.put((r, w, local, m))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 0, 20.0), (1, 2, 1, 20.0)]
