"""The autotuner's choice is a pure function of its timing table: the
smallest median wins, a value not clearly better than the current choice
loses to it, ties go to the smaller value, and coordinate descent over the
knobs gives the same parameters whatever order the trials are timed in.
The launch-parameter entry points refuse unknown names and values out of
range without a device."""
import ctypes
import random

import pytest

from vedas_gb300 import tune


def test_select_smallest_median_with_margin_and_ties():
    assert tune.select({16: [1.0, 1.2, 1.1], 8: [0.8, 0.9, 0.85]}, 16) == 8
    # within 2% of the best: the current value stays
    assert tune.select({16: [1.00, 1.00, 1.00], 8: [0.99, 0.99, 0.99]}, 16) == 16
    # tied medians, current not among them: the smaller value
    assert tune.select({4: [2.0], 2: [1.0], 8: [1.005]}, 6) == 2
    assert tune.select({}, 7) == 7


def test_descent_is_deterministic_from_a_fake_timing_table():
    # a fake device: a trial's time is a fixed function of the parameters
    cost = {"sort_items": {16: 3.0, 12: 2.5, 8: 2.0}, "sort_lookback": {1: 1.0, 4: 0.5},
            "join_small_rows": {256: 1.0, 64: 1.5, 0: 4.0},
            "write_small_rows": {1024: 2.0, 256: 2.0, 4096: 1.0, 0: 3.0},
            "unique_small_rows": {256: 1.0, 0: 1.01}, "write_blocks_per_sm": {5: 2.0, 8: 2.0, 4: 1.0, 2: 1.0}}

    def make(seed):
        rng = random.Random(seed)

        def measure(p):
            base = sum(cost[k][v] for k, v in p.items())
            return base * (1.0 + 0.001 * rng.random())      # tiny noise, far below the margin
        return measure

    results = [tune.descend(make(s), reps=3)[0] for s in range(5)]
    assert all(r == results[0] for r in results)
    assert results[0] == {"sort_items": 8, "sort_lookback": 4, "join_small_rows": 256, "write_small_rows": 4096,
                          "unique_small_rows": 256, "write_blocks_per_sm": 2}


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "t.json")
    tune.save("GPU X", "batch/t2^26/q2^12", {"params": {"sort_items": 8}}, path)
    tune.save("GPU X", "batch/t2^20/q2^8", {"params": {"sort_items": 16}}, path)
    assert tune.load("GPU X", "batch/t2^26/q2^12", path)["params"] == {"sort_items": 8}
    assert tune.load("GPU Y", "batch/t2^26/q2^12", path) is None
    assert tune.shape_class(100_000_000, 4096) == "batch/t2^26/q2^12"


def test_tune_entry_points_validate_without_device(built):
    import vedas_gb300 as vg
    L = vg.lib()
    v = ctypes.c_int64()
    assert L.vg_tune_set(None, b"sort_items", 8) == 1
    assert L.vg_tune_get(None, b"sort_items", ctypes.byref(v)) == 1
