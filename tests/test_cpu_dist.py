"""bench.py on CPU: the multi-replica path (two gloo ranks meet only at the
barriers and in the max/sum reductions of their step times and query counts;
no collective on the data path), and the reference arm's JSON line."""
import json
import os
import socket
import subprocess
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


def test_reference_arm_json_line_on_cpu(built):
    """bench.py --impl reference runs on the host cores alone: one JSON line
    with the contract's keys, on the same workload description as the GPU arm."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--triples", "200000",
                        "--entities", "20000", "--queries", "64", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "queries/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 1
    assert "200k-triple chain graph" in line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
