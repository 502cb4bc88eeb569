"""The multi-GPU mode of bench.py is independent replicas: one process per GPU, a gloo barrier
around the timed region, the time as the maximum over ranks and the work as the sum (no
data-path collective).  Here two CPU ranks (gloo, world size 2) run the same helpers."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    world, r, local, pg = bench.dist_setup()
    assert (world, r, local) == (2, rank, rank) and pg is not None
    bench.barrier(pg)
    t = bench.allreduce_max(pg, 1.0 + rank)        # each rank's elapsed time
    n = bench.allreduce_sum(pg, 10.0 * (rank + 1))  # each rank's commutators
    out.put((rank, t, n))
    pg.destroy_process_group()


def test_two_rank_replicas_aggregate():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 2.0, 30.0), (1, 2.0, 30.0)]
