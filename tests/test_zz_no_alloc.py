"""vg_join_noalloc: the join for callers that cannot allocate device memory.

Such callers (a host that has split all HBM among its own pools and forbids
libraries from calling cudaMalloc, or a serving thread that may only launch
work) call this entry point with their own input and output buffers; it keeps
its scratch in a fixed device array.  Its rows must equal vg_join's, on two
calls in a row (the second call sees the first call's leftover scratch).
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_LEFT_ROWS = 1 << 21


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


def _case(ctx, seed, nl, nr, keys, lcols, rcols):
    import vedas_gb300 as vg
    rng = np.random.Generator(np.random.PCG64(seed))
    lk = np.sort(rng.integers(0, keys, size=nl, dtype=np.uint32))
    rk = np.sort(rng.integers(0, keys, size=nr, dtype=np.uint32))
    lv = [rng.integers(0, 1 << 31, size=nl, dtype=np.uint32) for _ in range(lcols - 1)]
    rv = [rng.integers(0, 1 << 31, size=nr, dtype=np.uint32) for _ in range(rcols - 1)]
    return (vg.Relation.from_host(ctx, [lk] + lv), vg.Relation.from_host(ctx, [rk] + rv))


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


def test_noalloc_join_matches_vg_join_twice(ctx):
    import vedas_gb300 as vg
    L = _bind()
    cases = [(11, 300_000, 500_000, 20_000, 2, 3), (12, 70_001, 9_000, 50_000, 3, 1)]
    for seed, nl, nr, keys, lc, rc in cases:          # two calls in a row
        lrel, rrel = _case(ctx, seed, nl, nr, keys, lc, rc)
        want, _ = vg.join(ctx, lrel, rrel)
        st, rows, out = _noalloc_join(ctx, L, lrel, rrel, capacity=want.nrows + 17)
        assert st == 0, L.vg_noalloc_last_error()
        assert rows == want.nrows
        out.ir.nrows = rows
        for a, b in zip(out.to_host(), want.to_host()):
            np.testing.assert_array_equal(a, b)
        for r in (lrel, rrel, want, out):
            r.free()


def test_noalloc_join_limits(ctx):
    L = _bind()
    lrel, rrel = _case(ctx, 13, 4_000, 4_000, 100, 2, 2)
    # too small an output: the required count comes back, nothing is written
    st, rows, out = _noalloc_join(ctx, L, lrel, rrel, capacity=1)
    assert st == 7 and rows > 1
    out.free()
    # more left rows than the fixed scratch holds: refused before any launch
    big = ctypes.c_uint64()
    st = L.vg_join_noalloc(_ptrs(lrel), 2, MAX_LEFT_ROWS + 1, _ptrs(rrel), 2, rrel.nrows, None, 0,
                           ctypes.byref(big), ctx.stream)
    assert st == 7
    for r in (lrel, rrel):
        r.free()
