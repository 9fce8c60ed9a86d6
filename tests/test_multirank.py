"""The bench's multi-rank logic on CPU ranks (gloo, world size 2): every
rank runs its own replica, the step time is the max over ranks and the
throughput the sum of the ranks' work; the ensemble's members are split
over the ranks, each member on exactly one, and the totals summed."""

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


def _ensemble_rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, _ = bench.dist_env()
    d = bench.Dist(w, "gloo")
    # member i: 1000·(i + 1) nodes, as the ensemble's members differ in size
    members = [(i, 1000 * (i + 1)) for i in range(7)]
    mine = bench.member_share(members, r, w)
    nodes = d.sum(float(sum(n for _, n in mine)))
    count = d.sum(float(len(mine)))
    d.barrier()
    d.close()
    out.put((r, [i for i, _ in mine], nodes, count))


def test_ensemble_members_are_split_over_the_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ensemble_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    owned = [i for _, ids, _, _ in results for i in ids]
    assert sorted(owned) == list(range(7))  # every member on exactly one rank
    assert results[0][1] == [0, 2, 4, 6] and results[1][1] == [1, 3, 5]
    total = float(sum(1000 * (i + 1) for i in range(7)))
    assert all(nodes == total and count == 7.0 for _, _, nodes, count in results)
