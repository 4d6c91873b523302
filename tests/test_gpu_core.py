"""Parity of the CUDA path against the CPU oracle (bit-exact, integer IDs)."""
import numpy as np
import pytest

from oracle import oracle_py
from vedas_gb300 import workloads

pytestmark = pytest.mark.gpu

INDEX_ARRAYS = ["p_idx_values", "p_idx_offsets", "ps_s_idx_values", "ps_idx_offsets",
                "po_o_idx_values", "po_idx_offsets", "ps_data", "po_data", "pso_data", "pos_data"]
FULL_ARRAYS = ["s_idx_values", "s_idx_offsets", "sp_p_idx_values", "sp_idx_offsets",
               "so_o_idx_values", "so_idx_offsets", "o_idx_values", "o_idx_offsets", "os_data",
               "op_p_idx_values", "op_idx_offsets", "spo_data", "sop_data", "ops_data", "osp_data"]


def _same_result(res, ref):
    cols = res.columns()
    assert res.headers == ref.headers
    assert len(cols) == len(ref.columns)
    for a, b in zip(cols, ref.columns):
        np.testing.assert_array_equal(a, b)
    assert [r[:4] for r in res.log()] == [r[:4] for r in ref.log]


@pytest.mark.parametrize("n,subjects,full", [(1, 1, False), (5000, 300, False), (200_000, 10_000, False),
                                             (60_000, 2_000, True)])
def test_index_build_matches_oracle(ctx, n, subjects, full):
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=n, n_subjects=subjects, seed=3)
    ix = vg.Index(ctx, g.s, g.p, g.o, full=full)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o, full=full)
    for name in INDEX_ARRAYS + (FULL_ARRAYS if full else []):
        np.testing.assert_array_equal(ix.array(name), ref.array(name), err_msg=name)
    ix.close()


def test_radix_sort_via_swap_is_stable(ctx):
    import vedas_gb300 as vg
    rng = np.random.Generator(np.random.PCG64(7))
    for n in (1, 2, 4095, 4096, 4097, 100_000, 1_000_003):
        k = rng.integers(0, 50, size=n, dtype=np.uint32)            # heavy duplicates
        v = np.arange(n, dtype=np.uint32)
        w = rng.integers(0, 1 << 31, size=n, dtype=np.uint32)
        rel = vg.Relation.from_host(ctx, [v, k, w])
        vg.swap(ctx, rel, 1)                                       # key column 1 -> column 0
        got = rel.to_host()
        exp = oracle_py.sort_by_first([k, v, w])
        for a, b in zip(got, exp):
            np.testing.assert_array_equal(a, b)
        rel.free()


def test_sort_full_width_keys(ctx):
    import vedas_gb300 as vg
    rng = np.random.Generator(np.random.PCG64(8))
    k = rng.integers(0, 1 << 32, size=300_000, dtype=np.uint64).astype(np.uint32)
    rel = vg.Relation.from_host(ctx, [k])
    vg.swap(ctx, rel, 0)
    np.testing.assert_array_equal(rel.to_host()[0], np.sort(k))
    rel.free()


def test_sort_rows_lexicographic(ctx):
    import vedas_gb300 as vg
    rng = np.random.Generator(np.random.PCG64(9))
    cols = [rng.integers(0, 5, size=50_000, dtype=np.uint32) for _ in range(3)]
    rel = vg.Relation.from_host(ctx, cols)
    vg.sort_rows(ctx, rel)
    order = np.lexsort(cols[::-1])
    for a, c in zip(rel.to_host(), cols):
        np.testing.assert_array_equal(a, c[order])
    rel.free()


def test_unique_adjacent(ctx):
    import vedas_gb300 as vg
    rng = np.random.Generator(np.random.PCG64(10))
    for n in (1, 3, 2048, 2049, 70_001):
        a = rng.integers(0, 3, size=n, dtype=np.uint32)
        b = rng.integers(0, 2, size=n, dtype=np.uint32)
        rel = vg.Relation.from_host(ctx, [a, b])
        vg.unique(ctx, rel)
        keep = np.ones(n, dtype=bool)
        keep[1:] = (a[1:] != a[:-1]) | (b[1:] != b[:-1])
        got = rel.to_host()
        np.testing.assert_array_equal(got[0], a[keep])
        np.testing.assert_array_equal(got[1], b[keep])
        rel.free()


@pytest.mark.parametrize("nl,nr,keys", [(1, 1, 3), (1000, 5000, 50), (70_000, 90_000, 30_000),
                                        (5000, 300_000, 3),
                                        # windows of right keys larger than shared memory: lockstep
                                        # searches in global memory
                                        (20_000, 3_000_000, 1_000_000), (3, 2_000_000, 10),
                                        (50_000, 4_000_000, 1 << 31)])
def test_join_matches_oracle(ctx, nl, nr, keys):
    import vedas_gb300 as vg
    rng = np.random.Generator(np.random.PCG64(nl + nr))
    lk = np.sort(rng.integers(0, keys, size=nl, dtype=np.uint32))
    rk = np.sort(rng.integers(0, keys, size=nr, dtype=np.uint32))
    lv = rng.integers(0, 1 << 30, size=nl, dtype=np.uint32)
    rv = rng.integers(0, 1 << 30, size=nr, dtype=np.uint32)
    L = vg.Relation.from_host(ctx, [lk, lv])
    R = vg.Relation.from_host(ctx, [rk, rv])
    out, fl = vg.join(ctx, L, R)
    li, ri = oracle_py.inner_join(lk, rk)
    got = out.to_host()
    assert out.nrows == li.shape[0]
    np.testing.assert_array_equal(got[0], lk[li])
    np.testing.assert_array_equal(got[1], lv[li])
    np.testing.assert_array_equal(got[2], rv[ri])
    if li.shape[0]:
        assert fl == (lk[li[0]], lk[li[-1]])
    for r in (L, R, out):
        r.free()


def test_star_query_c1_small(ctx):
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=200_000, n_subjects=10_000, seed=0)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    q = workloads.star_query(3, 7)
    _same_result(ix.query(q), ref.query(q))
    ix.close()


@pytest.mark.parametrize("graph", ["star", "chain"])
def test_mixed_queries_match_oracle(ctx, graph):
    import vedas_gb300 as vg
    if graph == "star":
        g = workloads.graph_small_star(n=200_000, n_subjects=10_000, seed=1)
    else:
        g = workloads.graph_chain(n=300_000, n_entities=30_000, seed=1)
    qs = workloads.query_mix(g, 200, seed=2)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    checked = 0
    for q in qs:
        r = ref.query(q)
        if r.status != 0:
            with pytest.raises(vg.VgError):
                ix.query(q)
            continue
        _same_result(ix.query(q), r)
        checked += 1
    assert checked > 150
    ix.close()


def test_select_results_own_their_columns(ctx):
    """Selects read index slices without copying them; a select handed to the
    caller must still own (and free) every column, with the reference's rows."""
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=120_000, n_subjects=6_000, seed=12)
    used0 = ctx.memory()[0]
    ix = vg.Index(ctx, g.s, g.p, g.o)
    order = np.lexsort((g.o, g.s, g.p))            # PSO order
    ps, pso, pp = g.s[order], g.o[order], g.p[order]
    for p in (1, 5, 9):
        b, e = np.searchsorted(pp, p, "left"), np.searchsorted(pp, p, "right")
        # two variables, both used: (subject, object) rows of predicate p
        rel, _ = vg.select(ctx, ix, 3, p, index_pos=False, second_used=True)
        got = rel.to_host()
        np.testing.assert_array_equal(got[0], ps[b:e])
        np.testing.assert_array_equal(got[1], pso[b:e])
        rel.free()
        # second variable unused: the distinct subjects, in order
        rel, _ = vg.select(ctx, ix, 3, p, index_pos=False, second_used=False)
        sub = ps[b:e]
        keep = np.ones(sub.shape[0], dtype=bool)
        keep[1:] = sub[1:] != sub[:-1]
        np.testing.assert_array_equal(rel.to_host()[0], sub[keep])
        rel.free()
        # one variable: subjects of (?, p, o)
        o = int(pso[b + (e - b) // 2])
        rel, _ = vg.select(ctx, ix, 1, p, constant=o)
        exp = np.sort(g.s[(g.p == p) & (g.o == o)], kind="stable")
        np.testing.assert_array_equal(rel.to_host()[0], exp)
        rel.free()
    ix.close()
    assert ctx.memory()[0] == used0               # every column freed exactly once


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_waits_time_out_and_context_stays_usable(ctx, which):
    """A device wait that can never be satisfied gives up with a timeout
    status instead of hanging; the next work on the context runs normally."""
    import vedas_gb300 as vg
    st = vg.lib().vg_selfcheck_bounded_wait(ctx.h, which)
    assert st == 4                                   # VG_ERR_TIMEOUT
    g = workloads.graph_small_star(n=20_000, n_subjects=1_000, seed=30)
    ix = vg.Index(ctx, g.s, g.p, g.o)
    ref = oracle_py.OracleIndex(g.s, g.p, g.o)
    q = workloads.star_query(1, 2)
    _same_result(ix.query(q), ref.query(q))
    ix.close()
