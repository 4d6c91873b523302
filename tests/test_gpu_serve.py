"""Serving: queries admitted while others are in flight share waves, and
every result is the same as when the query runs alone."""
import threading
import time

import numpy as np
import pytest

from oracle import oracle_py
from vedas_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_results_alone_equal_results_in_the_mix(ctx):
    import vedas_gb300 as vg
    g = workloads.graph_chain(n=400_000, n_entities=40_000, seed=8)
    qs = workloads.query_mix(g, 240, seed=9, mix={"S": 0.6, "C": 0.3, "F": 0.1})
    ix = vg.Index(ctx, g.s, g.p, g.o)
    alone = {}
    for i, q in enumerate(qs):
        try:
            r = ix.query(q)
            alone[i] = (r.headers, r.columns())
            r.close()
        except vg.VgError:
            alone[i] = None
    srv = vg.Server(ix, budget_bytes=2 << 30)
    tickets = {}

    def client(part):
        for i in part:
            tickets[i] = srv.submit(qs[i])
            time.sleep(0.0005)          # staggered arrivals: queries join waves in flight

    def client_many(part):
        for c in range(0, len(part), 7):   # groups planned in parallel by submit_many
            chunk = part[c:c + 7]
            for i, t in zip(chunk, srv.submit_many([qs[i] for i in chunk])):
                tickets[i] = t
            time.sleep(0.001)

    th = [threading.Thread(target=client, args=(list(range(k, len(qs), 4)),)) for k in range(3)]
    th.append(threading.Thread(target=client_many, args=(list(range(3, len(qs), 4)),)))
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, t in tickets.items():
        assert srv.wait(t, 120.0)
        if alone[i] is None:
            assert srv.status(t) != 0
            continue
        assert srv.status(t) == 0
        heads, cols = alone[i]
        assert srv.headers(t) == heads
        for a, b in zip(srv.columns(t), cols):
            np.testing.assert_array_equal(a, b)
        q_s, tot_s = srv.latency(t)
        assert 0 <= q_s <= tot_s
        srv.release(t)
    st = srv.stats()
    assert st["completed"] + st["rejected"] == len(qs)
    assert st["peak_inflight"] > 1          # work of several queries overlapped
    srv.stop()
    ix.close()


def test_admission_rejects_over_budget_and_matches_oracle(ctx):
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=100_000, n_subjects=5_000, seed=10)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    srv = vg.Server(ix, budget_bytes=256 << 10)     # 256 KiB: the big star cannot fit
    big = workloads.star_query(1, 2)
    t_big = srv.submit(big)
    assert srv.wait(t_big, 30.0)
    assert srv.status(t_big) == 8                   # VG_ERR_REJECTED
    small = "SELECT ?x WHERE { ?x <5> <%d> . }" % int(g.o[np.nonzero(g.p == 5)[0][0]])
    t = srv.submit(small)
    assert srv.wait(t, 30.0) and srv.status(t) == 0
    r = ref.query(small)
    for a, b in zip(srv.columns(t), r.columns):
        np.testing.assert_array_equal(a, b)
    srv.release(t)
    srv.stop()
    ix.close()


def test_unreleased_results_hold_back_admission_without_stalling(ctx):
    """Finished results count against the budget until released: with a
    budget smaller than the results a client keeps, every query still
    finishes (the queue head is admitted whenever nothing is in flight), and
    releasing them lets the next ones in."""
    import vedas_gb300 as vg
    g = workloads.graph_chain(n=400_000, n_entities=40_000, seed=8)
    qs = workloads.query_mix(g, 64, seed=11, mix={"S": 0.6, "C": 0.3, "F": 0.1})
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    srv = vg.Server(ix, budget_bytes=1 << 20)        # 1 MiB: a few results fill it
    tickets = srv.submit_many([q.encode() for q in qs])
    for t in tickets:                                # nothing released while waiting
        assert srv.wait(t, 60.0)
    for q, t in zip(qs, tickets):
        r = ref.query(q)
        if r.status != 0 or srv.status(t) == 8:      # refused, or over the budget on its own
            continue
        assert srv.status(t) == 0, q
        for a, b in zip(srv.columns(t), r.columns):
            np.testing.assert_array_equal(a, b, err_msg=q)
    for t in tickets:
        srv.release(t)
    t = srv.submit(qs[0])
    assert srv.wait(t, 60.0)
    srv.release(t)
    srv.stop()
    ix.close()


def test_queue_limit_refuses_queries_that_waited_too_long(ctx):
    """Load shedding: with a small budget only a few queries run at a time,
    and those that waited in the queue longer than the limit are refused
    (VG_ERR_REJECTED); the admitted ones still match the oracle."""
    import vedas_gb300 as vg
    g = workloads.graph_chain(n=400_000, n_entities=40_000, seed=8)
    qs = workloads.query_mix(g, 400, seed=12, mix={"S": 0.6, "C": 0.3, "F": 0.1})
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    srv = vg.Server(ix, budget_bytes=1 << 20, queue_limit_s=0.002)
    tickets = srv.submit_many([q.encode() for q in qs])
    ok = shed = 0
    for q, t in zip(qs, tickets):
        assert srv.wait(t, 60.0)
        st = srv.status(t)
        if st == 0:
            ok += 1
            r = ref.query(q)
            for a, b in zip(srv.columns(t), r.columns):
                np.testing.assert_array_equal(a, b, err_msg=q)
        elif st == 8:
            shed += 1
        srv.release(t)
    assert ok > 0 and shed > 0, (ok, shed)
    srv.stop()
    ix.close()
