"""vg_join_noalloc: the join for callers that cannot allocate device memory.

Such callers (a host that has split all HBM among its own pools and forbids
libraries from calling cudaMalloc, or a serving thread that may only launch
work) call this entry point with their own input and output buffers; it keeps
its scratch in a fixed device array.  Its rows must equal the CPU oracle's
join (and vg_join's) on two calls in a row: the second call sees the first
call's leftover scratch.  The file is collected last so that a run stopping
at its first failure has run every other test already; it needs nothing from
them and passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_LEFT_ROWS = 1 << 21
VG_ERR_INVALID = 1
VG_ERR_OVERFLOW = 7


def _bind():
    import vedas_gb300 as vg
    L = vg.lib()
    fn = L.vg_join_noalloc
    pp = ctypes.POINTER(ctypes.c_void_p)
    fn.restype = ctypes.c_int
    fn.argtypes = [pp, ctypes.c_uint32, ctypes.c_uint64, pp, ctypes.c_uint32, ctypes.c_uint64, pp,
                   ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p]
    L.vg_noalloc_last_error.restype = ctypes.c_char_p
    return L


def _ptrs(rel, n=None):
    n = rel.ncols if n is None else n
    return (ctypes.c_void_p * n)(*[rel.ir.cols[c] for c in range(n)])


def _case(seed, nl, nr, keys, lcols, rcols):
    rng = np.random.Generator(np.random.PCG64(seed))
    lk = np.sort(rng.integers(0, keys, size=nl, dtype=np.uint32))
    rk = np.sort(rng.integers(0, keys, size=nr, dtype=np.uint32))
    lv = [rng.integers(0, 1 << 31, size=nl, dtype=np.uint32) for _ in range(lcols - 1)]
    rv = [rng.integers(0, 1 << 31, size=nr, dtype=np.uint32) for _ in range(rcols - 1)]
    return [lk] + lv, [rk] + rv


def _oracle_join(lh, rh):
    """Output columns of the reference's join (src/JoinQueryJob.cu:262-380):
    key, the left side's other columns, the right side's other columns, in
    (left row, right row) order; the pairs come from the CPU oracle."""
    from oracle import oracle_py
    li, ri = oracle_py.inner_join(lh[0], rh[0])
    return [lh[0][li]] + [c[li] for c in lh[1:]] + [c[ri] for c in rh[1:]]


def _noalloc_join(ctx, L, lrel, rrel, capacity):
    import vedas_gb300 as vg
    ncols = lrel.ncols + rrel.ncols - 1
    out = vg.vg_ir()
    vg.check(vg.lib().vg_ir_alloc(ctx.h, ncols, capacity, ctypes.byref(out)))
    outrel = vg.Relation(ctx, out)
    rows = ctypes.c_uint64()
    st = L.vg_join_noalloc(_ptrs(lrel), lrel.ncols, lrel.nrows, _ptrs(rrel), rrel.ncols, rrel.nrows,
                           _ptrs(outrel, ncols), capacity, ctypes.byref(rows), ctx.stream)
    return st, rows.value, outrel


def test_noalloc_join_matches_oracle_and_vg_join_twice(ctx):
    import vedas_gb300 as vg
    L = _bind()
    # the second case has fewer left rows than the first, so it runs over the
    # first call's leftover offsets and look-back words
    cases = [(11, 300_000, 500_000, 20_000, 2, 3), (12, 70_001, 9_000, 50_000, 3, 1)]
    for seed, nl, nr, keys, lc, rc in cases:          # two calls in a row
        lh, rh = _case(seed, nl, nr, keys, lc, rc)
        want = _oracle_join(lh, rh)
        lrel, rrel = vg.Relation.from_host(ctx, lh), vg.Relation.from_host(ctx, rh)
        st, rows, out = _noalloc_join(ctx, L, lrel, rrel, capacity=len(want[0]) + 17)
        assert st == 0, L.vg_noalloc_last_error()
        assert rows == len(want[0])
        out.ir.nrows = rows
        got = out.to_host()
        assert len(got) == len(want)
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)      # integer ids: bit-exact
        same, _ = vg.join(ctx, lrel, rrel)
        for a, b in zip(got, same.to_host()):
            np.testing.assert_array_equal(a, b)
        for r in (lrel, rrel, same, out):
            r.free()


def test_noalloc_join_limits(ctx):
    import vedas_gb300 as vg
    L = _bind()
    lh, rh = _case(13, 4_000, 4_000, 100, 2, 2)
    lrel, rrel = vg.Relation.from_host(ctx, lh), vg.Relation.from_host(ctx, rh)
    # too small an output: the required count comes back, nothing is written
    st, rows, out = _noalloc_join(ctx, L, lrel, rrel, capacity=1)
    assert st == VG_ERR_OVERFLOW and rows == len(_oracle_join(lh, rh)[0])
    out.free()
    # more left rows than the fixed scratch holds: refused before any launch
    big = ctypes.c_uint64()
    st = L.vg_join_noalloc(_ptrs(lrel), 2, MAX_LEFT_ROWS + 1, _ptrs(rrel), 2, rrel.nrows, None, 0,
                           ctypes.byref(big), ctx.stream)
    assert st == VG_ERR_OVERFLOW
    # column counts whose sum wraps around 32 bits: refused, nothing read
    st = L.vg_join_noalloc(_ptrs(lrel), 0xFFFFFFFF, lrel.nrows, _ptrs(rrel), 2, rrel.nrows, None, 0,
                           ctypes.byref(big), ctx.stream)
    assert st == VG_ERR_INVALID
    for r in (lrel, rrel):
        r.free()
