"""The N > 1 path of bench.py (replicas, one per GPU) on CPU: two gloo ranks
combine their step times as the bench does (slowest rank's time, elements of
all ranks)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 5.0 + rank  # rank 1 is the slower one
    res = bench.combine_ranks(dist, world, 1000, ms, 2 * ms, "cpu")
    out.put((rank, res))
    dist.destroy_process_group()


def test_two_rank_combination_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ms, e2e_ms, value, e2e = got[r]
        assert ms == 6.0 and e2e_ms == 12.0
        assert value == pytest.approx(2 * 1000 / 6e-3)
        assert e2e == pytest.approx(2 * 1000 / 12e-3)
