"""Batched multi-query execution: every query's result (headers, rows in
order, execution log) equals the oracle's and the one-query-at-a-time path's."""
import numpy as np
import pytest

from oracle import oracle_py
from vedas_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("graph,nq", [("star", 300), ("chain", 400)])
def test_batch_matches_oracle_and_plain(ctx, graph, nq):
    import vedas_gb300 as vg
    if graph == "star":
        g = workloads.graph_small_star(n=200_000, n_subjects=10_000, seed=4)
    else:
        g = workloads.graph_chain(n=400_000, n_entities=40_000, seed=4)
    qs = workloads.query_mix(g, nq, seed=5)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    b = vg.Batch(ix, qs)
    assert b.waves >= 1
    ok = 0
    for i, q in enumerate(qs):
        r = ref.query(q)
        if r.status != 0:
            assert b.status(i) != 0
            continue
        assert b.status(i) == 0, b.error(i)
        assert b.headers(i) == r.headers
        for a, c in zip(b.columns(i), r.columns):
            np.testing.assert_array_equal(a, c)
        assert [x[:4] for x in b.log(i)] == [x[:4] for x in r.log]
        ok += 1
    assert ok > 0.9 * nq
    # the same queries one at a time give the same rows
    for i in range(0, nq, 37):
        if b.status(i) != 0:
            continue
        res = ix.query(qs[i])
        for a, c in zip(res.columns(), b.columns(i)):
            np.testing.assert_array_equal(a, c)
    b.close()
    ix.close()


def test_batch_isolates_refused_queries(ctx):
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=20_000, n_subjects=1_000, seed=6)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    qs = [workloads.star_query(3, 7), "SELECT * WHERE { ?x ?p ?o . }", "not a query",
          workloads.star_query(2, 5)]
    b = vg.Batch(ix, qs)
    assert b.status(0) == 0 and b.status(3) == 0
    assert b.status(1) != 0 and b.status(2) != 0
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    for i in (0, 3):
        r = ref.query(qs[i])
        for a, c in zip(b.columns(i), r.columns):
            np.testing.assert_array_equal(a, c)
    b.close()
    ix.close()


def test_batch_empty_and_single(ctx):
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=5_000, n_subjects=500, seed=7)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    b = vg.Batch(ix, [])
    assert b.run() == 0
    b.close()
    q = workloads.star_query(1, 2)
    b = vg.Batch(ix, [q])
    r = oracle_py.OracleIndex(g.s, g.p, g.o).query(q)
    for a, c in zip(b.columns(0), r.columns):
        np.testing.assert_array_equal(a, c)
    b.close()
    ix.close()


def test_batch_host_copies_equal_device_results(ctx):
    """Results copied to host memory while the batch runs equal the device
    results, query by query, over two batches that reuse the host chunks."""
    import vedas_gb300 as vg
    g = workloads.graph_chain(n=300_000, n_entities=30_000, seed=14)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    for seed in (15, 16):
        qs = workloads.query_mix(g, 500, seed=seed)
        b = vg.Batch(ix, qs, to_host=True)
        plain = vg.Batch(ix, qs)
        total = 0
        for i in range(len(qs)):
            assert b.status(i) == plain.status(i)
            if b.status(i) != 0:
                continue
            dev = plain.columns(i)
            host = b.host_columns(i)
            assert len(dev) == len(host)
            for a, c in zip(host, dev):
                np.testing.assert_array_equal(a, c)
            total += sum(a.shape[0] for a in host)
        assert total > 0
        assert 4 * b.result_words() == 4 * plain.result_words()
        plain.close()
        b.close()
    ix.close()


@pytest.mark.parametrize("streams", ["1", "0"])
@pytest.mark.parametrize("region_mb", ["0", "1", "64"])
def test_batch_join_placement_regions(ctx, monkeypatch, region_mb, streams):
    """Join outputs placed on the device in a per-engine region (the default),
    in a region so small that most outputs overflow it and are written after a
    host round trip instead, and with no region at all; the wave engines on
    streams of their own (the default) or all on the context's stream: the
    same results and logs, and the arena holds no more than before once the
    batches are freed."""
    import vedas_gb300 as vg
    monkeypatch.setenv("VG_JOIN_REGION_MB", region_mb)
    monkeypatch.setenv("VG_ENGINE_STREAMS", streams)
    g = workloads.graph_chain(n=400_000, n_entities=40_000, seed=21)
    qs = workloads.query_mix(g, 400, seed=22)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    used0 = ctx.memory()[0]
    for _ in range(2):                      # a second batch reuses what the first one freed
        b = vg.Batch(ix, qs)
        for i, q in enumerate(qs):
            r = ref.query(q)
            if r.status != 0:
                assert b.status(i) != 0
                continue
            assert b.status(i) == 0, b.error(i)
            assert b.headers(i) == r.headers
            for a, c in zip(b.columns(i), r.columns):
                np.testing.assert_array_equal(a, c)
            assert [x[:4] for x in b.log(i)] == [x[:4] for x in r.log]
        b.close()
    assert ctx.memory()[0] == used0         # every region went back with its last output
    ix.close()


@pytest.mark.parametrize("params", [
    {"sort_items": 8, "sort_lookback": 1, "join_small_rows": 0, "write_small_rows": 0, "unique_small_rows": 0,
     "write_blocks_per_sm": 1},
    {"sort_items": 12, "sort_lookback": 4, "join_small_rows": 256, "write_small_rows": 1024,
     "unique_small_rows": 0, "write_blocks_per_sm": 5},
    {"sort_items": 16, "sort_lookback": 1, "join_small_rows": 64, "write_small_rows": 4096,
     "unique_small_rows": 256, "write_blocks_per_sm": 2},
])
def test_launch_parameters_change_speed_only(ctx, params):
    """Every autotuner choice (sort tile and look-back width, warp-per-join
    thresholds, write grid) gives the oracle's results, logs included, and the
    index build with the same sort choices gives the oracle's arrays."""
    import vedas_gb300 as vg
    from vedas_gb300 import tune
    g = workloads.graph_chain(n=300_000, n_entities=30_000, seed=31)
    qs = workloads.query_mix(g, 300, seed=32)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    old = {k: ctx.tune_get(k) for k in params}
    tune.apply(ctx, params)
    try:
        b = vg.Batch(ix, qs)
        for i, q in enumerate(qs):
            r = ref.query(q)
            if r.status != 0:
                assert b.status(i) != 0
                continue
            assert b.status(i) == 0, b.error(i)
            for a, c in zip(b.columns(i), r.columns):
                np.testing.assert_array_equal(a, c)
            assert [x[:4] for x in b.log(i)] == [x[:4] for x in r.log]
        b.close()
        # the index build's sort with the same tile choice
        ix2 = vg.Index(ctx, g.s, g.p, g.o)
        for name in ("ps_data", "pso_data", "po_data", "pos_data", "ps_idx_offsets", "po_idx_offsets"):
            np.testing.assert_array_equal(ix2.array(name), ref.array(name), err_msg=name)
        ix2.close()
    finally:
        tune.apply(ctx, old)
    ix.close()
