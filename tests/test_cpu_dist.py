"""The multi-replica path of bench.py on CPU: two gloo ranks meet only at the
barriers and in the max/sum reductions of their step times and query counts
(no collective on the data path)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    class A:
        pass
    r, w, loc, pg = bench.dist_setup(A())
    bench.barrier(pg)
    step_ms = 10.0 * (r + 1)                       # rank 1 is the slow one
    out[r] = (bench.max_over_ranks(pg, step_ms), bench.sum_over_ranks(pg, 4096.0), w, loc)
    bench.barrier(pg)
    pg.destroy_process_group()


def test_two_replicas_reduce_max_time_and_sum_queries():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    procs = [mp.get_context("spawn").Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        mx, total, w, loc = out[r]
        assert mx == 20.0 and total == 8192.0 and w == 2 and loc == r
