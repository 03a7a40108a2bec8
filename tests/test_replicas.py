"""The multi-rank side of bench.py on CPU (gloo, world size 2): one process per
rank, a barrier around the timed region, the slowest rank's time reported.
Each rank runs an independent replica (the single grid is not sharded), so
the only collective is this timing reduction."""
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


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      KG_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_init(world)
    bench.barrier(w)
    t = bench.max_over_ranks(1.5 + rank, w)
    bench.barrier(w)
    q.put((r, w, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_timing_reduction_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 2.5), (1, 2, 2.5)]
