#!/usr/bin/env python
"""VEDAS GB300 benchmark: the 4096-query mixed batch on the 100M-triple graph.

One step = every query of the batch run through the core (select, join and
index-swap kernels over the HBM-resident permutation indexes), results left
in HBM.  `value` is queries/s over all ranks; `e2e` is the same through the
C-ABI with every result downloaded to host memory inside the timed region.

--impl reference times the reference path's CPU implementation (this
project's restatement in oracle/, the reference's own build being x86-only
here) on the host cores, on a bounded sample of the same batch.

Multi-GPU: replicas only.  Every rank holds its own index and runs its own
4096-query batch (weak scaling); ranks meet only at the barriers around the
timed region.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched queries/s"
UNIT = "queries/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="batch", choices=["batch", "plain", "serve", "c3", "profile"],
                    help="batch: the 4096-query batch (default); plain: the same queries one at a "
                         "time; serve: Poisson arrivals on the hub graph; c3: the large snowflake "
                         "query on the 500M-triple hub graph; profile: index build and batches only, "
                         "for profilers")
    ap.add_argument("--rate", default="2000", help="serve: Poisson arrival rates (q/s), comma-separated")
    ap.add_argument("--clients", type=int, default=4, help="serve: submitter threads")
    ap.add_argument("--serve-pool", type=int, default=20000, help="serve: distinct queries drawn from")
    ap.add_argument("--duration", type=float, default=10.0, help="serve: seconds of arrivals")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="serve: relation memory budget")
    ap.add_argument("--queue-limit-ms", type=float, default=0.0,
                    help="serve: refuse queries that waited longer in the queue (0: no limit)")
    ap.add_argument("--triples", type=int, default=None,
                    help="graph size (default: 100M; 500M for --mode c3 and serve)")
    ap.add_argument("--entities", type=int, default=None,
                    help="entities (default: 2M; 10M for --mode c3 and serve)")
    ap.add_argument("--queries", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=256, help="queries per CPU-baseline step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ingest-triples", type=int, default=20_000_000,
                    help="triples of the N-Triples ingest measurement (0: skip)")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default launch parameters (no autotuner trials)")
    ap.add_argument("--arena-gb", type=float, default=0.0,
                    help="HBM arena size (0: 90%% of free memory; profilers need room to replay)")
    a = ap.parse_args()
    hub = a.mode in ("c3", "serve")
    if a.triples is None:
        a.triples = 500_000_000 if hub else 100_000_000
    if a.entities is None:
        a.entities = 10_000_000 if hub else 2_000_000
    return a


T_START = time.perf_counter()


def note(msg: str) -> None:
    """Progress line on stderr (stdout carries only the JSON line)."""
    print(f"[bench {time.perf_counter() - T_START:7.1f}s] {msg}", file=sys.stderr, flush=True)


def triples_label(n: int) -> str:
    """100000000 -> '100M', 200000 -> '200k'."""
    if n % 1_000_000 == 0:
        return f"{n // 1_000_000}M"
    if n % 1_000 == 0:
        return f"{n // 1_000}k"
    return str(n)


# ---------------------------------------------------------------------------
def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    local_world = int(os.environ.get("LOCAL_WORLD_SIZE", str(world)))
    if local_world > 1 and "VG_HOST_THREADS" not in os.environ:
        # replicas on one node share its cores: each process's host worker
        # threads (read once, when the library makes its pools) get a share
        cpus = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        os.environ["VG_HOST_THREADS"] = str(max(2, cpus // local_world))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        for row in csv.reader(io.StringIO(out)):
            if len(row) < 9:
                continue
            try:
                sm.append(float(row[1]))
                smax.append(float(row[2]))
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for nm, v in zip(names, row[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def traffic_table():
    """DRAM bytes (read + write) per launch of each kernel, averaged over every
    launch of the kernel in one ncu capture of this bench's default command
    (every batched step runs the same batch, so each step launches the same
    work); written by hand from that capture's summary in profiles/."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(p) as f:
            return {k: float(v["dram_bytes_per_launch"]) for k, v in json.load(f).items()}
    except (OSError, ValueError, KeyError, TypeError):
        return {}


# ---------------------------------------------------------------------------
def make_workload(args, rank: int):
    from vedas_gb300 import workloads
    g = workloads.graph_chain(n=args.triples, n_entities=args.entities, seed=args.seed)
    cs = workloads.ConstantSampler(g)
    queries = workloads.query_mix(g, args.queries, seed=args.seed + 1000 * rank, cs=cs)
    return g, queries, cs


def run_plain(ix, queries, download=False):
    """The reference's one-query-at-a-time loop (vdBench), on the GPU core."""
    import vedas_gb300 as vg
    rows = 0
    d2h = 0
    for q in queries:
        r = ix.query(q)
        rows += r.nrows
        if download:
            for c in r.columns():
                d2h += c.nbytes
        r.close()
    return rows, d2h


def run_batch(ix, queries, download=False, profile=None):
    """One batched step; with download every result also lands in host
    memory (copied while the batch runs, complete when it returns)."""
    import vedas_gb300 as vg
    b = vg.Batch(ix, queries, to_host=download)
    rows = b.run()
    d2h = 0
    if download:
        d2h = 4 * b.result_words()
    if profile is not None:
        for k, v in b.profile().items():
            profile[k] = profile.get(k, 0.0) + v
    b.close()
    return rows, d2h


def plain_latencies(ix, queries):
    """One pass of the one-query-at-a-time loop (the reference's vdBench
    pattern), run in C by vg_query_loop: wall time of the pass and per-query
    latencies."""
    t_all = time.perf_counter()
    sec, _, _ = ix.query_loop(queries)
    return time.perf_counter() - t_all, list(sec)


def cpu_baseline_run(g, queries, sample: int, steps: int = 1):
    """Times the oracle port (all host threads) on `sample` queries."""
    from oracle import oracle_py
    ox = oracle_py.OracleIndex(g.s, g.p, g.o)
    qs = queries[:sample]
    for q in qs[: min(8, len(qs))]:
        ox.query(q)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        for q in qs:
            ox.query(q)
        times.append(time.perf_counter() - t0)
    return len(qs), times, os.cpu_count()


def batch_config(args, nq: int, world: int) -> dict:
    """The workload both arms report (the reference arm times a sample of it)."""
    return {"workload": f"{nq}-query mixed batch (20 star/chain/snowflake templates, "
                        f"1-8 patterns) on the {triples_label(args.triples)}-triple chain graph",
            "mode": "batch", "triples": args.triples, "entities": args.entities, "queries": nq,
            "parallelism": f"replicas{world}", "l2": "inputs larger than L2"}


def bench_reference(args, rank, world, pg):
    if rank != 0:
        return
    g, queries, _ = make_workload(args, 0)
    n, times, cores = cpu_baseline_run(g, queries, args.cpu_sample, steps=args.warmup + args.steps)
    timed = times[args.warmup:] if len(times) > args.warmup else times
    total = sum(timed)
    value = n * len(timed) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(timed),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded generator, no dataset)",
        "config": dict(batch_config(args, len(queries), world),
                       sample_queries_per_step=n),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} queries of the batch per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_ingest(args, ctx, g):
    """N-Triples ingest on the device (parse + dictionary encoding) of the
    first ingest_triples triples of the graph written as N-Triples text;
    wall time of the call (text upload, kernels, dictionary terms to the
    host) and kernel time, beside the CPU restatement on a sample."""
    import vedas_gb300 as vg
    from vedas_gb300 import workloads
    m = min(args.ingest_triples, g.n)
    sub = workloads.Graph(g.s[:m], g.p[:m], g.o[:m])
    text = workloads.to_ntriples(sub)
    vg.ingest_ntriples(ctx, text).free()          # warm-up
    ctx.stats_reset(timing=True)
    ctx.sync()
    t0 = time.perf_counter()
    ing = vg.ingest_ntriples(ctx, text)
    wall = time.perf_counter() - t0
    st = ctx.stats()
    ing.free()
    ctx.stats_reset(timing=False)
    kms = sum(v[2] for v in st.values())
    out = {"triples": m, "text_bytes": len(text), "wall_ms": 1000 * wall, "triples_per_s": m / wall,
           "text_GBps": len(text) / wall / 1e9, "device_ms": kms,
           "dictionary": {"so": ing.dict.size("so"), "p": ing.dict.size("p")},
           "kernels": {k: round(v[2], 3) for k, v in st.items() if k.startswith("ingest") or k.startswith("radix")}}
    if not args.no_cpu_baseline:
        from oracle import oracle_py
        k = min(m, 2_000_000)
        t1 = time.perf_counter()
        oracle_py.ingest_ntriples(text[:101 * k])
        out["cpu_oracle_triples_per_s"] = k / (time.perf_counter() - t1)
        out["cpu_oracle_sample"] = f"{k} triples, one thread (the loader's sequential hash-map rule)"
    return out


def bench_profile(args, local):
    """For profilers: the index build (from device columns, inside an NVTX
    start/end range named index_build) and then only --warmup + --steps
    batches of the workload, the timed ones inside a start/end range named
    timed_batch (ncu --nvtx --nvtx-include timed_batch).  Start/end ranges are
    process-wide, so they hold the launches of every wave engine's thread.
    Prints the step time, which is not a reported number."""
    import torch
    import vedas_gb300 as vg
    g, queries, _ = make_workload(args, 0)
    ctx = vg.Context(local, arena_bytes=int(args.arena_gb * (1 << 30)))
    dcols = [torch.from_numpy(x.astype(np.int32)).cuda(local) for x in (g.s, g.p, g.o)]
    torch.cuda.synchronize(local)
    r_build = torch.cuda.nvtx.range_start("index_build")
    ix = vg.Index(ctx, device_ptrs=[c.data_ptr() for c in dcols], n=g.n)
    ctx.sync()
    torch.cuda.nvtx.range_end(r_build)
    del dcols
    batch_in = [q.encode() for q in queries]
    for _ in range(args.warmup):
        run_batch(ix, batch_in)
    ctx.sync()
    r_batch = torch.cuda.nvtx.range_start("timed_batch")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run_batch(ix, batch_in)
    ctx.sync()
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    torch.cuda.nvtx.range_end(r_batch)
    print(json.dumps({"mode": "profile", "triples": g.n, "queries": len(queries), "s_per_step": dt}), flush=True)
    ix.close()
    ctx.close()


def bench_ours(args, rank, world, local, pg):
    import torch
    import vedas_gb300 as vg
    from vedas_gb300 import workloads as wl

    g, queries, cs = make_workload(args, rank)
    note(f"workload: {g.n} triples, {len(queries)} queries")
    ctx = vg.Context(local, arena_bytes=int(args.arena_gb * (1 << 30)))
    t0 = time.perf_counter()
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ctx.sync()
    build_s = time.perf_counter() - t0
    # index build on device-resident columns, kernels timed with CUDA events
    build = None
    import torch
    dcols = [torch.from_numpy(x.astype(np.int32)).cuda(local) for x in (g.s, g.p, g.o)]
    torch.cuda.synchronize(local)
    ctx.stats_reset(timing=True)
    ix2 = vg.Index(ctx, device_ptrs=[c.data_ptr() for c in dcols], n=g.n)
    kst = ctx.stats()
    ix2.close()
    del dcols
    kms = sum(v[2] for v in kst.values())
    if kms > 0:
        build = {"triples": g.n, "device_ms": kms, "rows_per_s": g.n / (kms / 1000.0),
                 "algorithmic_GBps": 2 * 24.0 * g.n / (kms / 1000.0) / 1e9,
                 "kernels": {k: round(v[2], 3) for k, v in kst.items()}}
    note("index built")
    ingest = bench_ingest(args, ctx, g) if args.ingest_triples > 0 else None
    note("ingest leg done")
    chain = None
    try:
        cq = wl.chain_query(g, cs=cs)
        ix.query(cq).close()
        ts = []
        for _ in range(5):
            ctx.sync()
            t1 = time.perf_counter()
            r = ix.query(cq)
            ts.append(time.perf_counter() - t1)
            rows = r.nrows
            log = r.log()
            r.close()
        chain = {"query": cq, "rows": rows, "ms_min": 1000 * min(ts), "ms_median": 1000 * float(np.median(ts)),
                 "log": [list(x) for x in log]}
        oq = wl.chain_query_open()
        ix.query(oq).close()
        ts = []
        for _ in range(5):
            ctx.sync()
            t1 = time.perf_counter()
            r = ix.query(oq)
            ts.append(time.perf_counter() - t1)
            orows = r.nrows
            olog = r.log()
            r.close()
        chain["open_end"] = {"query": oq, "rows": orows, "ms_min": 1000 * min(ts),
                             "ms_median": 1000 * float(np.median(ts)), "log": [list(x) for x in olog]}
    except vg.VgError as e:
        chain = {"error": str(e)}
    # The core refuses queries on which the reference itself would read out of
    # bounds or trip an assert; drop those before timing (counted below).
    note("chain queries done")
    b = vg.Batch(ix, queries)
    kept = [q for i, q in enumerate(queries) if b.status(i) == 0]
    qrows = b.rows()
    b.close()
    # share of each template's instances that return rows
    nt = len(wl.TEMPLATES)
    nonempty = [round(float(np.mean([qrows[i] > 0 for i in range(k, len(queries), nt)])), 3) for k in range(nt)]
    refused = len(queries) - len(kept)
    run = run_batch if args.mode == "batch" else run_plain
    # the batch API takes UTF-8 query text; encode it once, as a client would
    batch_in = [q.encode() for q in kept] if args.mode == "batch" else kept
    tuned = None
    if not args.no_tune:
        from vedas_gb300 import tune
        tuned = tune.tune_batch(ix, [q.encode() for q in kept], reps=3, triples=g.n)
        note(f"launch parameters: {tuned['params']} ({'cached' if tuned['from_cache'] else 'tuned'})")
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)

    for _ in range(args.warmup):
        run(ix, batch_in)
    note("batch warm-up done")
    plain_s, plain_lat = plain_latencies(ix, kept)
    note("plain loop done")
    plain = {"queries_per_s": len(kept) / plain_s,
             "p50_ms": 1000 * float(np.percentile(plain_lat, 50)),
             "p99_ms": 1000 * float(np.percentile(plain_lat, 99))}
    prof = {}
    # L2 (129 MB) is far smaller than the 100M-triple index (2.4 GB of data
    # columns), so consecutive steps do not reuse each other's lines.
    clocks = ClockSampler(local)
    ctx.stats_reset(timing=False)        # launches are counted; no per-kernel events in the timed steps
    barrier(pg)
    ctx.sync()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    rows = 0
    for _ in range(args.steps):
        r, _ = run(ix, batch_in, profile=prof) if args.mode == "batch" else run(ix, kept)
        rows += r
    ev1.record(stream)
    ctx.sync()
    clk = clocks.stop()
    barrier(pg)
    step_ms = ev0.elapsed_time(ev1) / args.steps
    launches = ctx.launches()
    step_ms_max = max_over_ranks(pg, step_ms)
    total_q = sum_over_ranks(pg, float(len(kept)))
    value = total_q / (step_ms_max / 1000.0)

    note("timed batch steps done")
    # end to end: results copied to host memory inside the timed region (after
    # warm-up steps of the same path: page-locked result buffers are made once)
    for _ in range(args.warmup):
        run(ix, batch_in, download=True)
    ctx.stats_reset(timing=False)
    barrier(pg)
    ctx.sync()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(args.steps):
        _, b = run(ix, batch_in, download=True)
        d2h += b
    ctx.sync()
    e2e_s = max_over_ranks(pg, (time.perf_counter() - t0) / args.steps)
    e2e_value = total_q / e2e_s
    note("end-to-end steps done")
    h2d = sum(len(q) for q in kept)
    stats = kernel_pass(ctx, lambda: run(ix, batch_in), args.steps)

    peak, peak_kind = peak_hbm()
    dom = max(stats.items(), key=lambda kv: kv[1][2]) if stats else None
    roof = None
    if dom:
        name, (n_l, bytes_, ms) = dom
        achieved = bytes_ / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
        tr = traffic_table().get(name)
        roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": f"of {peak_kind}",
                "traffic": tr,
                "algorithmic_bytes_per_launch": bytes_ / max(n_l, 1), "launches": n_l,
                "avg_launch_us": 1000.0 * ms / max(n_l, 1)}
    kernels = {k: {"launches": v[0], "ms": round(v[2], 3), "GBps": round(v[1] / v[2] / 1e6, 1) if v[2] else None}
               for k, v in stats.items()}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n, times, cores = cpu_baseline_run(g, kept, args.cpu_sample)
        cpu = {"value": n / times[-1], "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"first {n} queries of the batch, oracle restatement on host cores"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded generator, no dataset)",
            "config": dict(batch_config(args, len(kept), world), mode=args.mode, queries_refused=refused,
                           result_rows_per_step=rows // max(args.steps, 1), index_build_s=round(build_s, 3),
                           template_nonempty_share=nonempty),
            "result_rows_per_s": rows / max(args.steps, 1) / (step_ms_max / 1000.0),
            "roofline": roof,
            "plain_per_query": plain,
            "speedup_vs_plain": value / (world * plain["queries_per_s"]),
            "batch_latency_ms": {"p50": step_ms_max, "p99": step_ms_max,
                                 "note": "every query of a batch completes with the batch"},
            "host_device_split_s_per_step": {k: round(v / args.steps, 4) for k, v in prof.items()},
            "launch_parameters": tuned,
            "index_build": build,
            "chain_query": chain,
            "ingest": ingest,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h // max(args.steps, 1)},
            "gpu_launches": launches,
            "clocks": clk,
            "kernels": kernels,
            "kernel_timing": f"CUDA events per launch over {args.steps} more steps with every engine on one stream",
        }
        print(json.dumps(line), flush=True)
    ix.close()
    ctx.close()


def dedup_on_device(g, device: int):
    """The triples made a set (sorted by p, s, o), deduplicated with torch on
    the device; input preparation outside every timed region."""
    import torch
    from vedas_gb300 import workloads
    bs = int(g.s.max()).bit_length()
    bo = int(g.o.max()).bit_length()
    key = (torch.from_numpy(g.p.astype(np.int64)) << (bs + bo)) | (torch.from_numpy(g.s.astype(np.int64)) << bo) \
        | torch.from_numpy(g.o.astype(np.int64))
    u = torch.unique(key.cuda(device)).cpu().numpy()
    del key
    torch.cuda.empty_cache()
    o = (u & ((1 << bo) - 1)).astype(np.uint32)
    s = ((u >> bo) & ((1 << bs) - 1)).astype(np.uint32)
    p = (u >> (bs + bo)).astype(np.uint32)
    return workloads.Graph(s, p, o, g.name + "_set")


def kernel_pass(ctx, step, steps):
    """Per-kernel launches, algorithmic bytes and CUDA-event milliseconds
    over `steps` more steps with every wave engine on the context's stream
    (VG_ENGINE_STREAMS=0): kernels then run one after another, so each event
    pair brackets its own kernel only.  With the engines on their own streams
    (the timed steps) a pair would also span the other streams' kernels."""
    old = os.environ.get("VG_ENGINE_STREAMS")
    os.environ["VG_ENGINE_STREAMS"] = "0"
    try:
        ctx.sync()
        ctx.stats_reset(timing=True)
        for _ in range(steps):
            step()
        ctx.sync()
        st = ctx.stats()
        ctx.stats_reset(timing=False)
    finally:
        if old is None:
            os.environ.pop("VG_ENGINE_STREAMS", None)
        else:
            os.environ["VG_ENGINE_STREAMS"] = old
    return st


def roofline_of(stats):
    """Roofline entry of the kernel with the most device time."""
    peak, peak_kind = peak_hbm()
    if not stats:
        return None
    name, (n_l, bytes_, ms) = max(stats.items(), key=lambda kv: kv[1][2])
    achieved = bytes_ / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
    return {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": f"of {peak_kind}", "traffic": traffic_table().get(name),
            "algorithmic_bytes_per_launch": bytes_ / max(n_l, 1), "launches": n_l,
            "avg_launch_us": 1000.0 * ms / max(n_l, 1)}


def bench_c3(args, rank, world, local, pg):
    """The large single query: the seven-pattern snowflake on the 500M-triple
    hub graph (relations of about 1.6e8 rows, a result of about 4.6e8 rows x
    8 columns).  One step = one vg_query with the result left in HBM;
    `value` is result rows/s; e2e adds the download of every result column to
    page-locked host memory."""
    import torch
    import vedas_gb300 as vg
    from vedas_gb300 import workloads
    g = dedup_on_device(workloads.graph_hub(n=args.triples, n_entities=args.entities, seed=args.seed,
                                            dedup=False), local)
    q = workloads.snowflake_query(workloads.C3_SNOWFLAKE)
    ctx = vg.Context(local, arena_bytes=int(args.arena_gb * (1 << 30)))
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    rows = 0
    for _ in range(args.warmup):
        r = ix.query(q)
        rows = r.nrows
        log = r.log()
        r.close()
    clocks = ClockSampler(local)
    ctx.stats_reset(timing=True)
    barrier(pg)
    ctx.sync()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        r = ix.query(q)
        rows = r.nrows
        r.close()
    ev1.record(stream)
    ctx.sync()
    clk = clocks.stop()
    barrier(pg)
    stats = ctx.stats()
    launches = ctx.launches()
    step_ms = max_over_ranks(pg, ev0.elapsed_time(ev1) / args.steps)
    total_rows = sum_over_ranks(pg, float(rows))
    # end to end: the same query, every result column copied to pinned host memory
    ctx.stats_reset(timing=False)
    ncols = 8
    host = torch.empty((ncols, max(rows, 1)), dtype=torch.int32, pin_memory=True)
    e2e = []
    for it in range(args.warmup + args.steps):
        ctx.sync()
        t0 = time.perf_counter()
        r = ix.query(q)
        for c in range(ncols):
            r.download_into(c, host[c].data_ptr())
        r.close()
        if it >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(pg, float(np.mean(e2e)))
    if rank == 0:
        line = {
            "metric": "large-query result rows/s", "value": total_rows / (step_ms / 1000.0), "unit": "rows/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": f"seven-pattern snowflake {workloads.C3_SNOWFLAKE} on the "
                                   f"{triples_label(args.triples)}-triple hub graph",
                       "mode": "c3", "triples": g.n, "entities": args.entities, "result_rows": rows,
                       "result_cols": ncols, "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2", "query": q},
            "execution_log": [list(x) for x in log],
            "roofline": roofline_of(stats),
            "e2e": {"value": total_rows / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": len(q),
                    "d2h_bytes_per_step": 4 * rows * ncols, "ms_per_step": 1000 * e2e_s},
            "gpu_launches": launches,
            "clocks": clk,
            "kernels": {k: {"launches": v[0], "ms": round(v[2], 3),
                            "GBps": round(v[1] / v[2] / 1e6, 1) if v[2] else None} for k, v in stats.items()},
        }
        print(json.dumps(line), flush=True)
    ix.close()
    ctx.close()


def serve_point(srv, qb, rate, duration, clients, seed):
    """One offered rate: Poisson arrivals over `duration` seconds, split over
    `clients` submitter threads (arrival i goes to thread i % clients); each
    thread submits its due queries in one call and hands the tickets to a
    collector of its own, which waits for each result and releases it (the
    server counts unreleased results against its memory budget, as a client
    that reads its results and lets go of them).  A query's latency runs from
    its scheduled arrival to its completion."""
    import queue as _queue
    n_q = int(rate * duration)
    rng = np.random.Generator(np.random.PCG64(seed))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n_q))
    picks = rng.integers(0, len(qb), size=n_q)
    late = np.zeros(n_q)
    status = np.zeros(n_q, dtype=np.int64)
    total = np.zeros(n_q)
    inbox = [_queue.SimpleQueue() for _ in range(clients)]
    t0 = time.perf_counter()

    def client(c):
        mine = np.arange(c, n_q, clients)
        k = 0
        while k < len(mine):
            now = time.perf_counter() - t0
            if arrivals[mine[k]] > now:
                time.sleep(min(arrivals[mine[k]] - now, 0.0005))
                continue
            e = k + int(np.searchsorted(arrivals[mine[k:]], now, side="right"))
            idx = mine[k:e]
            sub = time.perf_counter() - t0
            ts = srv.submit_many([qb[j] for j in picks[idx]])
            late[idx] = sub - arrivals[idx]
            inbox[c].put((idx, ts))
            k = e
        inbox[c].put(None)

    def collector(c):
        while True:
            item = inbox[c].get()
            if item is None:
                return
            for i, t in zip(*item):
                srv.wait(t)
                status[i] = srv.status(t)
                total[i] = srv.latency(t)[1]
                srv.release(t)

    th = [threading.Thread(target=client, args=(c,)) for c in range(clients)]
    th += [threading.Thread(target=collector, args=(c,)) for c in range(clients)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.perf_counter() - t0
    okm = status == 0
    lat = total[okm] + np.maximum(late[okm], 0.0)
    ok = int(okm.sum())
    statuses = {}
    for st in status[~okm]:
        statuses[int(st)] = statuses.get(int(st), 0) + 1
    return {"offered_rate": rate, "queries": n_q, "served_rate": ok / wall, "completed": ok,
            "failed_or_rejected": n_q - ok, "failure_statuses": {str(k): v for k, v in sorted(statuses.items())},
            "wall_s": wall,
            "latency_ms": {"p50": 1000 * float(np.percentile(lat, 50)), "p95": 1000 * float(np.percentile(lat, 95)),
                           "p99": 1000 * float(np.percentile(lat, 99))}}


def bench_serve(args, rank, world, local, pg):
    """Serving: the hub graph resident in HBM, Poisson arrivals from several
    client threads, continuous batching with memory-budget admission;
    p50/p95/p99 latency and sustained queries/s over all ranks (replicas) at
    each offered rate (--rate, comma-separated: the first is the headline)."""
    import vedas_gb300 as vg
    from vedas_gb300 import workloads
    rates = [float(x) for x in str(args.rate).split(",")]
    g = dedup_on_device(workloads.graph_hub(n=args.triples, n_entities=args.entities, seed=args.seed,
                                            dedup=False), local)
    note(f"hub graph: {g.n} triples")
    cs = workloads.ConstantSampler(g)
    # a pool of instantiated queries with the 60/30/10 star/chain/snowflake mix
    pool = workloads.query_mix(g, args.serve_pool, seed=args.seed + 7 + 1000 * rank, cs=cs,
                               mix={"S": 0.6, "C": 0.3, "F": 0.1})
    qb = [q.encode() for q in pool]
    note(f"{len(pool)} queries instantiated")
    ctx = vg.Context(local, arena_bytes=int(args.arena_gb * (1 << 30)))
    ix = vg.Index(ctx, g.s, g.p, g.o)
    del g, cs
    srv = vg.Server(ix, budget_bytes=int(args.budget_gb * (1 << 30)), queue_limit_s=args.queue_limit_ms / 1000.0)
    for t in srv.submit_many(qb[:256]):     # warm-up: first waves, host mirrors
        srv.wait(t)
        srv.release(t)
    points = []
    for k, rate in enumerate(rates):
        barrier(pg)
        pt = serve_point(srv, qb, rate, args.duration, args.clients, args.seed + 99 + rank + 17 * k)
        pt["served_rate"] = sum_over_ranks(pg, pt["served_rate"])
        points.append(pt)
        note(f"rate {rate:.0f}: served {pt['served_rate']:.0f} q/s, p50 {pt['latency_ms']['p50']:.2f} ms, "
             f"p99 {pt['latency_ms']['p99']:.2f} ms")
    stats = srv.stats()
    srv.stop()
    if rank == 0:
        head = points[0]
        line = {
            "metric": "serving queries/s", "value": head["served_rate"], "unit": UNIT, "n_gpus": world,
            "higher_is_better": True, "scaling": "weak", "dtype": "u32",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": f"Poisson arrivals at {rates[0]:.0f} q/s for {args.duration:.0f} s from "
                                   f"{args.clients} client threads, 60/30/10 star/chain/snowflake templates, on "
                                   f"the {triples_label(args.triples)}-triple hub graph",
                       "budget_gb": args.budget_gb, "query_pool": len(pool), "clients": args.clients,
                       "queue_limit_ms": args.queue_limit_ms or None,
                       "waves": stats["waves"], "peak_inflight": stats["peak_inflight"]},
            "latency_ms": head["latency_ms"],
            "offered_rate": rates[0],
            "points": points,
        }
        print(json.dumps(line), flush=True)
    ix.close()
    ctx.close()


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args)
    if args.impl == "reference":
        bench_reference(args, rank, world, pg)
    elif args.mode == "serve":
        bench_serve(args, rank, world, local, pg)
    elif args.mode == "c3":
        bench_c3(args, rank, world, local, pg)
    elif args.mode == "profile":
        bench_profile(args, local)
    else:
        bench_ours(args, rank, world, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
