#!/usr/bin/env python
"""Calibrates the CPU baseline: the reference's own query path (the
reference sources compiled for the host, oracle/_ref/vedas_ref) against this
project's restatement (oracle/liboracle.so), timed on the same queries of
the benchmark batch, on the same graph, with the same OpenMP thread count.

Test infrastructure only (it runs the two checkers, nothing of the product).
Needs oracle/_ref/vedas_ref, which exists only where the reference sources
were available to build it.

  python oracle/calibrate_cpu.py [--triples 100000000] [--queries 256] [--reps 3]

Prints one JSON line: seconds per pass of each, queries/s of each and the
ratio restatement / reference (above 1: the restatement is faster).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--triples", type=int, default=100_000_000)
    ap.add_argument("--entities", type=int, default=None)
    ap.add_argument("--queries", type=int, default=256)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    a = ap.parse_args()
    os.environ["OMP_NUM_THREADS"] = str(a.threads)
    from oracle import oracle_py, ref_runner
    from vedas_gb300 import workloads
    if not ref_runner.available():
        sys.exit("oracle/_ref/vedas_ref is not built (make -C oracle ref REF=<reference checkout>)")
    ent = a.entities or max(1, a.triples // 50)
    g = workloads.graph_chain(n=a.triples, n_entities=ent, seed=0)
    # the first queries of the benchmark batch (same generator, seed and order)
    qs = workloads.query_mix(g, 4096, seed=0)[:a.queries]
    with tempfile.TemporaryDirectory() as td:
        gp = os.path.join(td, "g.bin")
        qp = os.path.join(td, "q.txt")
        g.save(gp)
        with open(qp, "w") as f:
            f.write("\n".join(qs) + "\n")
        err = subprocess.run([ref_runner.REF_BIN, "time", gp, qp, str(a.reps)], check=True,
                             capture_output=True, text=True, cwd=td).stderr
    times = [ln.split() for ln in err.splitlines() if ln.startswith("TIME ")]
    ref_s = [float(t[2]) for t in times]
    ref_rows = int(times[-1][3])
    ox = oracle_py.OracleIndex(g.s, g.p, g.o)
    for q in qs:                                    # untimed pass, as for the reference
        ox.query(q)
    port_s, port_rows = [], 0
    for _ in range(a.reps):
        t0 = time.perf_counter()
        port_rows = 0
        for q in qs:
            port_rows += ox.query(q).nrows
        port_s.append(time.perf_counter() - t0)
    line = {"triples": g.n, "queries": len(qs), "threads": a.threads,
            "reference_s_per_pass": ref_s, "restatement_s_per_pass": port_s,
            "reference_queries_per_s": len(qs) / min(ref_s), "restatement_queries_per_s": len(qs) / min(port_s),
            "restatement_over_reference": min(ref_s) / min(port_s),
            "result_rows": {"reference": ref_rows, "restatement": port_rows}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
