"""The bench's multi-rank logic on CPU ranks (gloo, world size 2): every
rank runs its own replica, the step time is the max over ranks and the
throughput the sum of the ranks' work."""

import os
import socket
import sys
from pathlib import Path

import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, local = bench.dist_env()
    d = bench.Dist(w, "gloo")
    d.barrier()
    seconds = d.max(1.0 + r)        # rank 1 is the slow one
    nodes = d.sum(1000.0 * (r + 1))
    d.close()
    out.put((r, local, seconds, nodes))


def test_two_ranks_take_the_slowest_time_and_all_the_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert results == [(0, 0, 2.0, 3000.0), (1, 1, 2.0, 3000.0)]
