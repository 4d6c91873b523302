"""Autotuner for the core's launch parameters (vg_tune_set).

The kernels' launch shapes have choices whose best value depends on the GPU
and on the workload's shape (relation sizes, how many queries run together):
radix-sort keys per thread (the sort tile) and look-back words loaded at
once, the sizes below which a join, a
join output or a final compaction takes one warp instead of tiles, and the
block count of a join write sized on the device.  No choice changes a result.

tune_batch() picks them from timed trials of a batch: coordinate descent in
a fixed knob order, each candidate value timed `reps` times with the others
at their current choice, the smallest median winning.  Values within
`margin` of the best median tie; the current choice wins a tie, else the
smallest value, so the selection is a pure function of the timing table
(select()) and noise below the margin cannot change it.  Choices are cached in a JSON
file keyed by GPU name and shape class (VG_TUNE_CACHE, default
~/.cache/vedas_gb300/tune.json).
"""
from __future__ import annotations

import json
import math
import os
import statistics
import time

# knob -> (candidate values, value of a fresh context)
KNOBS = {
    "sort_items": ([16, 12, 8], 16),
    "sort_lookback": ([4, 1], 4),
    "join_small_rows": ([256, 64, 0], 256),
    "write_small_rows": ([1024, 256, 4096, 0], 1024),
    "unique_small_rows": ([256, 0], 256),
    "write_blocks_per_sm": ([5, 8, 4, 2], 5),
}
ORDER = ["sort_items", "sort_lookback", "join_small_rows", "write_small_rows", "unique_small_rows", "write_blocks_per_sm"]


def select(timings: dict, current, margin: float = 0.02):
    """The value to keep given {value: [seconds, ...]}.  Values whose median
    is within `margin` (relative) of the smallest median tie: the current
    value if it is one of them, else the smallest of them.  Timing noise
    below the margin thus never changes the choice."""
    med = {v: statistics.median(ts) for v, ts in timings.items() if ts}
    if not med:
        return current
    best = min(med.values())
    tied = [v for v, m in med.items() if m <= best * (1.0 + margin)]
    return current if current in tied else min(tied)


def shape_class(triples: int, queries: int) -> str:
    """Workloads whose graph and batch sizes share their power-of-two bucket
    share their choices."""
    def b(x):
        return int(math.log2(max(1, x)))
    return f"batch/t2^{b(triples)}/q2^{b(queries)}"


def gpu_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001 - torch is optional here
        pass
    return "unknown-gpu"


def cache_path() -> str:
    return os.environ.get("VG_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "vedas_gb300",
                                                          "tune.json")


def load(gpu: str, shape: str, path: str | None = None):
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f).get(gpu, {}).get(shape)
    except (OSError, ValueError):
        return None


def save(gpu: str, shape: str, entry: dict, path: str | None = None) -> None:
    path = path or cache_path()
    data = {}
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        pass
    data.setdefault(gpu, {})[shape] = entry
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def descend(measure, reps: int = 3, knobs=None, order=None, margin: float = 0.02):
    """Coordinate descent: measure(params) -> seconds of one trial.  Returns
    (chosen params, {knob: {value: [seconds, ...]}})."""
    knobs = knobs or KNOBS
    order = order or [k for k in ORDER if k in knobs]
    params = {k: knobs[k][1] for k in order}
    table = {}
    for k in order:
        cands, _ = knobs[k]
        timings = {}
        for v in cands:
            trial = dict(params, **{k: v})
            timings[v] = [measure(trial) for _ in range(reps)]
        params[k] = select(timings, params[k], margin)
        table[k] = timings
    return params, table


def apply(ctx, params: dict) -> None:
    for k, v in params.items():
        ctx.tune_set(k, v)


def tune_batch(ix, queries, reps: int = 3, triples: int = 0, use_cache: bool = True, write_cache: bool = True):
    """Chooses the launch parameters for batches like `queries` on index
    `ix` (cached per GPU and shape class), applies them to ix's context and
    returns {"gpu", "shape", "params", "from_cache", "trials"}."""
    import vedas_gb300 as vg
    ctx = ix.ctx
    gpu = gpu_name()
    shape = shape_class(triples, len(queries))
    if use_cache:
        hit = load(gpu, shape)
        if hit and set(hit.get("params", {})) == set(KNOBS):
            apply(ctx, hit["params"])
            return {"gpu": gpu, "shape": shape, "params": hit["params"], "from_cache": True, "trials": 0}
    qb = [q if isinstance(q, bytes) else q.encode() for q in queries]
    trials = [0]

    def measure(p):
        apply(ctx, p)
        ctx.sync()
        t0 = time.perf_counter()
        b = vg.Batch(ix, qb)
        ctx.sync()
        dt = time.perf_counter() - t0
        b.close()
        trials[0] += 1
        return dt

    measure({k: v[1] for k, v in KNOBS.items()})          # warm-up trial
    params, table = descend(measure, reps=reps)
    apply(ctx, params)
    entry = {"params": params,
             "medians_ms": {k: {str(v): round(1000 * statistics.median(ts), 3) for v, ts in t.items()}
                            for k, t in table.items()}}
    if write_cache:
        save(gpu, shape, entry)
    return {"gpu": gpu, "shape": shape, "params": params, "from_cache": False, "trials": trials[0],
            "medians_ms": entry["medians_ms"]}
