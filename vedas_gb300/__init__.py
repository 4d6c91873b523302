"""VEDAS query-execution core for GB300 (sm_103a), Python bindings.

The product is the in-tree shared library ``libvedas_gb300.so`` (CUDA kernels
plus the host-side mirror of the reference's query path) behind the C-ABI in
``include/vedas_gb300.h``.  This module only binds that ABI with ctypes; it
raises if the library is missing rather than falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvedas_gb300.so")
MAX_COLS = 9

_lib = None


class VgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


STATUS = {0: "ok", 1: "invalid", 2: "oom", 3: "cuda", 4: "timeout", 5: "unsupported",
          6: "parse", 7: "overflow", 8: "rejected"}


class vg_ir(ctypes.Structure):
    _fields_ = [("ncols", ctypes.c_uint32), ("nrows", ctypes.c_uint64),
                ("cols", ctypes.c_void_p * MAX_COLS)]


class vg_select_desc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("index_pos", ctypes.c_int), ("pred", ctypes.c_uint32),
                ("constant", ctypes.c_uint32), ("has_bound", ctypes.c_int),
                ("bound_lo", ctypes.c_uint32), ("bound_hi", ctypes.c_uint32),
                ("eif", ctypes.c_uint64 * 4), ("second_used", ctypes.c_int)]


def lib():
    """Loads the library (it must have been built by __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        pu32 = ctypes.POINTER(u32)
        sigs = {
            "vg_status_string": (ctypes.c_char_p, [i32]),
            "vg_last_error": (ctypes.c_char_p, []),
            "vg_ctx_create": (i32, [i32, ctypes.c_size_t, ctypes.POINTER(vp)]),
            "vg_ctx_destroy": (i32, [vp]),
            "vg_ctx_memory": (i32, [vp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t),
                                    ctypes.POINTER(ctypes.c_size_t)]),
            "vg_ctx_sync": (i32, [vp]),
            "vg_ctx_stream": (vp, [vp]),
            "vg_stats_reset": (i32, [vp, i32]),
            "vg_stats_count": (u32, [vp]),
            "vg_stats_launches": (u64, [vp]),
            "vg_stats_get": (i32, [vp, u32, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(u64),
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
            "vg_index_build": (i32, [vp, vp, vp, vp, u64, i32, i32, ctypes.POINTER(vp)]),
            "vg_index_free": (i32, [vp]),
            "vg_index_array": (i32, [vp, ctypes.c_char_p, ctypes.POINTER(vp), ctypes.POINTER(pu32),
                                     ctypes.POINTER(u64)]),
            "vg_index_write": (i32, [vp, ctypes.c_char_p]),
            "vg_index_open": (i32, [vp, ctypes.c_char_p, i32, ctypes.POINTER(vp)]),
            "vg_ir_alloc": (i32, [vp, u32, u64, ctypes.POINTER(vg_ir)]),
            "vg_ir_free": (i32, [vp, ctypes.POINTER(vg_ir)]),
            "vg_ir_upload": (i32, [vp, ctypes.POINTER(vg_ir), u32, pu32, u64]),
            "vg_ir_download": (i32, [vp, ctypes.POINTER(vg_ir), u32, pu32]),
            "vg_select": (i32, [vp, vp, ctypes.POINTER(vg_select_desc), ctypes.POINTER(vg_ir), pu32]),
            "vg_join": (i32, [vp, ctypes.POINTER(vg_ir), ctypes.POINTER(vg_ir), ctypes.POINTER(vg_ir), pu32]),
            "vg_join2": (i32, [vp, ctypes.POINTER(vg_ir), ctypes.POINTER(vg_ir), ctypes.POINTER(vg_ir)]),
            "vg_swap": (i32, [vp, ctypes.POINTER(vg_ir), u32]),
            "vg_sort_rows": (i32, [vp, ctypes.POINTER(vg_ir)]),
            "vg_unique": (i32, [vp, ctypes.POINTER(vg_ir)]),
            "vg_eif_scan": (i32, [vp, ctypes.POINTER(vg_ir), ctypes.POINTER(u64)]),
            "vg_query": (i32, [vp, vp, ctypes.c_char_p, ctypes.POINTER(vp)]),
            "vg_result_ncols": (u32, [vp]),
            "vg_result_nrows": (u64, [vp]),
            "vg_result_header": (ctypes.c_char_p, [vp, u32]),
            "vg_result_column_device": (vp, [vp, u32]),
            "vg_result_download": (i32, [vp, u32, pu32]),
            "vg_result_nlog": (u32, [vp]),
            "vg_result_log": (None, [vp, u32, pu32, ctypes.POINTER(u64), ctypes.POINTER(u64),
                                     ctypes.POINTER(u64)]),
            "vg_result_free": (i32, [vp]),
            "vg_tune_set": (i32, [vp, ctypes.c_char_p, ctypes.c_int64]),
            "vg_tune_get": (i32, [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]),
            "vg_query_loop": (i32, [vp, vp, ctypes.POINTER(ctypes.c_char_p), u32, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(u64), ctypes.POINTER(i32)]),
            "vg_batch_run": (i32, [vp, vp, ctypes.POINTER(ctypes.c_char_p), u32, ctypes.POINTER(vp)]),
            "vg_batch_run_host": (i32, [vp, vp, ctypes.POINTER(ctypes.c_char_p), u32, ctypes.POINTER(vp)]),
            "vg_batch_host_column": (vp, [vp, u32, u32]),
            "vg_batch_size": (u32, [vp]),
            "vg_batch_waves": (u32, [vp]),
            "vg_batch_query_status": (i32, [vp, u32]),
            "vg_batch_query_error": (ctypes.c_char_p, [vp, u32]),
            "vg_batch_ncols": (u32, [vp, u32]),
            "vg_batch_nrows": (u64, [vp, u32]),
            "vg_batch_rows": (i32, [vp, vp]),
            "vg_batch_header": (ctypes.c_char_p, [vp, u32, u32]),
            "vg_batch_column_device": (vp, [vp, u32, u32]),
            "vg_batch_download": (i32, [vp, u32, u32, pu32]),
            "vg_batch_result_words": (u64, [vp]),
            "vg_batch_download_all": (i32, [vp, vp]),
            "vg_batch_profile": (i32, [vp, ctypes.POINTER(ctypes.c_double)]),
            "vg_batch_nlog": (u32, [vp, u32]),
            "vg_batch_log": (None, [vp, u32, u32, pu32, ctypes.POINTER(u64), ctypes.POINTER(u64),
                                    ctypes.POINTER(u64)]),
            "vg_batch_free": (i32, [vp]),
            "vg_serve_start": (i32, [vp, vp, ctypes.c_size_t, ctypes.POINTER(vp)]),
            "vg_serve_submit": (i32, [vp, ctypes.c_char_p, ctypes.POINTER(u64)]),
            "vg_ingest_ntriples": (i32, [vp, ctypes.c_char_p, u64, ctypes.c_int, ctypes.POINTER(vp),
                                         ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(u64),
                                         ctypes.POINTER(vp)]),
            "vg_ingest_free": (i32, [vp, vp, vp, vp]),
            "vg_dict_size": (u64, [vp, ctypes.c_int]),
            "vg_dict_term": (ctypes.c_char_p, [vp, ctypes.c_int, u32]),
            "vg_dict_lookup": (u32, [vp, ctypes.c_int, ctypes.c_char_p]),
            "vg_dict_write": (i32, [vp, ctypes.c_char_p]),
            "vg_dict_open": (i32, [ctypes.c_char_p, ctypes.POINTER(vp)]),
            "vg_dict_free": (i32, [vp]),
            "vg_index_set_dict": (i32, [vp, vp]),
            "vg_result_decode": (i32, [vp, vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
            "vg_batch_decode": (i32, [vp, u32, vp, ctypes.c_char_p, ctypes.c_size_t,
                                      ctypes.POINTER(ctypes.c_size_t)]),
            "vg_ingest_set_hash_bits": (None, [ctypes.c_int]),
            "vg_selfcheck_bounded_wait": (i32, [vp, ctypes.c_int]),
            "vg_selfcheck_pools": (i32, [u32, u32, u32, ctypes.POINTER(u64)]),
            "vg_selfcheck_l2_lookup": (i32, [u32, u32, u32, ctypes.POINTER(u64)]),
            "vg_serve_submit_many": (i32, [vp, ctypes.POINTER(ctypes.c_char_p), u32, ctypes.POINTER(ctypes.c_uint64)]),
            "vg_serve_wait": (i32, [vp, u64, ctypes.c_double, ctypes.POINTER(i32)]),
            "vg_serve_query_status": (i32, [vp, u64]),
            "vg_serve_ncols": (u32, [vp, u64]),
            "vg_serve_nrows": (u64, [vp, u64]),
            "vg_serve_header": (ctypes.c_char_p, [vp, u64, u32]),
            "vg_serve_download": (i32, [vp, u64, u32, pu32]),
            "vg_serve_latency": (i32, [vp, u64, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double)]),
            "vg_serve_release": (i32, [vp, u64]),
            "vg_serve_set_queue_limit": (i32, [vp, ctypes.c_double]),
            "vg_serve_stats": (i32, [vp, ctypes.POINTER(u64)]),
            "vg_serve_stop": (i32, [vp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise VgError(status, f"{STATUS.get(status, status)}: {lib().vg_last_error().decode()}")


def _p32(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


class Context:
    """One device, one stream, one HBM arena (vg_ctx)."""

    def __init__(self, device: int = 0, arena_bytes: int = 0):
        h = ctypes.c_void_p()
        check(lib().vg_ctx_create(device, arena_bytes, ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().vg_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def tune_set(self, name: str, value: int) -> None:
        """Sets one launch parameter (vg_tune_set)."""
        check(lib().vg_tune_set(self.h, name.encode(), int(value)))

    def tune_get(self, name: str) -> int:
        v = ctypes.c_int64()
        check(lib().vg_tune_get(self.h, name.encode(), ctypes.byref(v)))
        return int(v.value)

    def memory(self):
        u, p, c = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        check(lib().vg_ctx_memory(self.h, ctypes.byref(u), ctypes.byref(p), ctypes.byref(c)))
        return u.value, p.value, c.value

    def sync(self):
        check(lib().vg_ctx_sync(self.h))

    @property
    def stream(self) -> int:
        return lib().vg_ctx_stream(self.h) or 0

    def stats_reset(self, timing: bool = False) -> None:
        check(lib().vg_stats_reset(self.h, int(timing)))

    def launches(self) -> int:
        return int(lib().vg_stats_launches(self.h))

    def stats(self) -> dict:
        """{kernel: (launches, algorithmic bytes, total ms)} since the last reset."""
        L = lib()
        out = {}
        for i in range(L.vg_stats_count(self.h)):
            name = ctypes.c_char_p()
            n, b, ms = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double()
            check(L.vg_stats_get(self.h, i, ctypes.byref(name), ctypes.byref(n), ctypes.byref(b),
                                 ctypes.byref(ms)))
            out[name.value.decode()] = (n.value, b.value, ms.value)
        return out


class Index:
    """Resident permutation indexes (VedasStorage layout)."""

    def __init__(self, ctx: Context, s=None, p=None, o=None, full: bool = False, handle=None,
                 device_ptrs=None, n: int = 0):
        self.ctx = ctx
        if handle is not None:
            self.h = handle
            return
        h = ctypes.c_void_p()
        if device_ptrs is not None:
            ds, dp, do = device_ptrs
            check(lib().vg_index_build(ctx.h, ds, dp, do, n, int(full), 1, ctypes.byref(h)))
        else:
            s, p, o = (np.ascontiguousarray(x, dtype=np.uint32) for x in (s, p, o))
            check(lib().vg_index_build(ctx.h, s.ctypes.data, p.ctypes.data, o.ctypes.data,
                                       s.shape[0], int(full), 0, ctypes.byref(h)))
        self.h = h

    @staticmethod
    def open(ctx: Context, path: str, full: bool = False) -> "Index":
        h = ctypes.c_void_p()
        check(lib().vg_index_open(ctx.h, path.encode(), int(full), ctypes.byref(h)))
        return Index(ctx, handle=h)

    def write(self, path: str) -> None:
        check(lib().vg_index_write(self.h, path.encode()))

    def set_dict(self, d) -> None:
        """Query constants as IRIs / literals through the dictionary d
        (None: numeric <ID> constants again)."""
        check(lib().vg_index_set_dict(self.h, d.h if d is not None else None))

    def close(self):
        if getattr(self, "h", None):
            lib().vg_index_free(self.h)
            self.h = None

    def array(self, name: str) -> np.ndarray:
        host = ctypes.POINTER(ctypes.c_uint32)()
        n = ctypes.c_uint64()
        check(lib().vg_index_array(self.h, name.encode(), None, ctypes.byref(host), ctypes.byref(n)))
        if n.value == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.ctypeslib.as_array(host, shape=(n.value,)).copy()

    def device_array(self, name: str):
        d = ctypes.c_void_p()
        n = ctypes.c_uint64()
        check(lib().vg_index_array(self.h, name.encode(), ctypes.byref(d), None, ctypes.byref(n)))
        return d.value, n.value

    def query(self, sparql: str) -> "Result":
        r = ctypes.c_void_p()
        check(lib().vg_query(self.ctx.h, self.h, sparql.encode(), ctypes.byref(r)))
        return Result(r)

    def query_loop(self, queries):
        """The queries one at a time in a C loop (vg_query_loop): per-query
        wall seconds, result rows and status as numpy arrays."""
        n = len(queries)
        arr, keep = _pack_texts(queries)
        sec = np.zeros(n, dtype=np.float64)
        rows = np.zeros(n, dtype=np.uint64)
        st = np.zeros(n, dtype=np.int32)
        check(lib().vg_query_loop(self.ctx.h, self.h, arr, n,
                                  sec.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  rows.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                  st.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        del keep
        return sec, rows, st


class Result:
    OPS = {0: "JOIN", 1: "UPLOAD", 2: "SWAP"}

    def __init__(self, h):
        self.h = h

    def __del__(self):
        self.close()

    def close(self):
        if getattr(self, "h", None):
            lib().vg_result_free(self.h)
            self.h = None

    @property
    def headers(self):
        L = lib()
        return [L.vg_result_header(self.h, c).decode() for c in range(L.vg_result_ncols(self.h))]

    @property
    def nrows(self) -> int:
        return int(lib().vg_result_nrows(self.h))

    def column(self, c: int) -> np.ndarray:
        """One result column, copied to host memory."""
        n = self.nrows
        a = np.zeros(n, dtype=np.uint32)
        if n:
            check(lib().vg_result_download(self.h, c, _p32(a)))
        return a

    def columns(self):
        return [self.column(c) for c in range(lib().vg_result_ncols(self.h))]

    def download_into(self, c: int, host_ptr: int) -> None:
        """Copies column c to host memory at host_ptr (nrows uint32 words)."""
        if self.nrows:
            check(lib().vg_result_download(self.h, c, ctypes.cast(host_ptr, ctypes.POINTER(ctypes.c_uint32))))

    def log(self):
        L = lib()
        recs = []
        for i in range(L.vg_result_nlog(self.h)):
            op, p1, p2, p3 = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
            L.vg_result_log(self.h, i, ctypes.byref(op), ctypes.byref(p1), ctypes.byref(p2), ctypes.byref(p3))
            recs.append((self.OPS[op.value], p1.value, p2.value, p3.value))
        return recs


def _pack_texts(queries):
    """The queries as a C array of NUL-terminated strings (const char**),
    built from one joined buffer; the second value keeps the buffer alive."""
    qb = [q if isinstance(q, bytes) else q.encode() for q in queries]
    n = len(qb)
    blob = np.frombuffer(b"\0".join(qb) + b"\0", dtype=np.uint8)
    lens = np.fromiter(map(len, qb), dtype=np.uint64, count=n)
    offs = np.zeros(n, dtype=np.uint64)
    if n > 1:
        np.cumsum(lens[:-1] + 1, out=offs[1:])
    ptrs = offs + np.uint64(blob.ctypes.data)
    return ptrs.ctypes.data_as(ctypes.POINTER(ctypes.c_char_p)), (blob, ptrs)


class Batch:
    """Many queries executed together (vg_batch_run)."""

    OPS = Result.OPS

    def __init__(self, ix: "Index", queries, to_host: bool = False):
        """Runs the queries; with to_host every result is also copied to
        page-locked host memory while the batch runs (host_columns)."""
        self.ix = ix
        self.n = len(queries)
        self.to_host = to_host
        arr, self._keep = _pack_texts(queries)
        h = ctypes.c_void_p()
        run = lib().vg_batch_run_host if to_host else lib().vg_batch_run
        check(run(ix.ctx.h, ix.h, arr, self.n, ctypes.byref(h)))
        self.h = h

    def host_columns(self, q: int):
        """Query q's result columns from the batch's host copies (to_host)."""
        if not self.to_host:
            raise VgError(1, "the batch was run without host copies")
        L = lib()
        n = self.nrows(q)
        out = []
        for c in range(L.vg_batch_ncols(self.h, q)):
            p = L.vg_batch_host_column(self.h, q, c)
            if n == 0 or not p:
                out.append(np.zeros(n, dtype=np.uint32))
            else:
                buf = (ctypes.c_uint32 * n).from_address(p)
                out.append(np.frombuffer(buf, dtype=np.uint32).copy())
        return out

    def run(self) -> int:
        """Total result rows (the batch already ran in the constructor)."""
        return int(self.rows().sum())

    def rows(self) -> np.ndarray:
        """Row count of every query (one call)."""
        out = np.zeros(self.n, dtype=np.uint64)
        if self.n:
            check(lib().vg_batch_rows(self.h, out.ctypes.data))
        return out

    @property
    def waves(self) -> int:
        return int(lib().vg_batch_waves(self.h))

    def status(self, q: int) -> int:
        return int(lib().vg_batch_query_status(self.h, q))

    def error(self, q: int) -> str:
        return lib().vg_batch_query_error(self.h, q).decode()

    def headers(self, q: int):
        L = lib()
        return [L.vg_batch_header(self.h, q, c).decode() for c in range(L.vg_batch_ncols(self.h, q))]

    def nrows(self, q: int) -> int:
        return int(lib().vg_batch_nrows(self.h, q))

    def columns(self, q: int):
        L = lib()
        n = self.nrows(q)
        out = []
        for c in range(L.vg_batch_ncols(self.h, q)):
            a = np.zeros(n, dtype=np.uint32)
            if n:
                check(L.vg_batch_download(self.h, q, c, _p32(a)))
            out.append(a)
        return out

    def result_words(self) -> int:
        return int(lib().vg_batch_result_words(self.h))

    def download_all(self, host_ptr: int) -> int:
        """Copies every result column into host memory at host_ptr (one copy);
        returns the number of bytes copied."""
        words = self.result_words()
        if words:
            check(lib().vg_batch_download_all(self.h, ctypes.c_void_p(host_ptr)))
        return 4 * words

    def profile(self) -> dict:
        """Host/device time split of the run, in seconds."""
        out = (ctypes.c_double * 6)()
        check(lib().vg_batch_profile(self.h, out))
        keys = ["plan_s", "prepare_s", "device_s", "finish_s", "final_s", "total_s"]
        return dict(zip(keys, list(out)))

    def log(self, q: int):
        L = lib()
        recs = []
        for i in range(L.vg_batch_nlog(self.h, q)):
            op, p1, p2, p3 = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
            L.vg_batch_log(self.h, q, i, ctypes.byref(op), ctypes.byref(p1), ctypes.byref(p2), ctypes.byref(p3))
            recs.append((self.OPS[op.value], p1.value, p2.value, p3.value))
        return recs

    def close(self):
        if getattr(self, "h", None):
            lib().vg_batch_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Server:
    """Continuous-batching serving loop (vg_serve_*)."""

    def __init__(self, ix: "Index", budget_bytes: int, queue_limit_s: float = 0.0):
        h = ctypes.c_void_p()
        check(lib().vg_serve_start(ix.ctx.h, ix.h, budget_bytes, ctypes.byref(h)))
        self.h = h
        if queue_limit_s:
            self.set_queue_limit(queue_limit_s)

    def set_queue_limit(self, seconds: float) -> None:
        """Queries that waited more than `seconds` in the queue are refused
        (status VG_ERR_REJECTED); 0 admits every query."""
        check(lib().vg_serve_set_queue_limit(self.h, ctypes.c_double(seconds)))

    def submit(self, sparql: str) -> int:
        t = ctypes.c_uint64()
        check(lib().vg_serve_submit(self.h, sparql.encode(), ctypes.byref(t)))
        return t.value

    def submit_many(self, queries) -> list:
        """Submits many queries at once (planned in parallel); their tickets."""
        n = len(queries)
        if n == 0:
            return []
        arr, keep = _pack_texts(queries)
        out = (ctypes.c_uint64 * n)()
        check(lib().vg_serve_submit_many(self.h, arr, n, out))
        return list(out)

    def wait(self, ticket: int, timeout_s: float = -1.0) -> bool:
        done = ctypes.c_int()
        check(lib().vg_serve_wait(self.h, ticket, timeout_s, ctypes.byref(done)))
        return bool(done.value)

    def status(self, ticket: int) -> int:
        return int(lib().vg_serve_query_status(self.h, ticket))

    def headers(self, ticket: int):
        L = lib()
        return [L.vg_serve_header(self.h, ticket, c).decode() for c in range(L.vg_serve_ncols(self.h, ticket))]

    def columns(self, ticket: int):
        L = lib()
        n = int(L.vg_serve_nrows(self.h, ticket))
        out = []
        for c in range(L.vg_serve_ncols(self.h, ticket)):
            a = np.zeros(n, dtype=np.uint32)
            if n:
                check(L.vg_serve_download(self.h, ticket, c, _p32(a)))
            out.append(a)
        return out

    def latency(self, ticket: int):
        q, t = ctypes.c_double(), ctypes.c_double()
        check(lib().vg_serve_latency(self.h, ticket, ctypes.byref(q), ctypes.byref(t)))
        return q.value, t.value

    def release(self, ticket: int) -> None:
        check(lib().vg_serve_release(self.h, ticket))

    def stats(self) -> dict:
        out = (ctypes.c_uint64 * 6)()
        check(lib().vg_serve_stats(self.h, out))
        keys = ["submitted", "completed", "rejected", "waves", "reserved_bytes", "peak_inflight"]
        return dict(zip(keys, [int(x) for x in out]))

    def stop(self) -> None:
        if getattr(self, "h", None):
            lib().vg_serve_stop(self.h)
            self.h = None

    def __del__(self):
        self.stop()


class Relation:
    """A device relation (vg_ir) owned by a context."""

    def __init__(self, ctx: Context, ir: vg_ir):
        self.ctx = ctx
        self.ir = ir

    @staticmethod
    def from_host(ctx: Context, cols) -> "Relation":
        cols = [np.ascontiguousarray(c, dtype=np.uint32) for c in cols]
        ir = vg_ir()
        n = cols[0].shape[0] if cols else 0
        check(lib().vg_ir_alloc(ctx.h, len(cols), n, ctypes.byref(ir)))
        for i, c in enumerate(cols):
            check(lib().vg_ir_upload(ctx.h, ctypes.byref(ir), i, _p32(c), n))
        return Relation(ctx, ir)

    @property
    def nrows(self) -> int:
        return int(self.ir.nrows)

    @property
    def ncols(self) -> int:
        return int(self.ir.ncols)

    def to_host(self):
        out = []
        for c in range(self.ir.ncols):
            a = np.zeros(self.ir.nrows, dtype=np.uint32)
            check(lib().vg_ir_download(self.ctx.h, ctypes.byref(self.ir), c, _p32(a)))
            out.append(a)
        return out

    def free(self):
        if self.ir.ncols:
            check(lib().vg_ir_free(self.ctx.h, ctypes.byref(self.ir)))


def select(ctx: Context, ix: Index, kind: int, pred: int, constant: int = 0, index_pos: bool = False,
           bound=None, eif=(0, 0, 0, 0), second_used: bool = True):
    d = vg_select_desc()
    d.kind, d.index_pos, d.pred, d.constant = kind, int(index_pos), pred, constant
    if bound is not None:
        d.has_bound, d.bound_lo, d.bound_hi = 1, bound[0], bound[1]
    for i in range(4):
        d.eif[i] = eif[i]
    d.second_used = int(second_used)
    out = vg_ir()
    bu = (ctypes.c_uint32 * 3)()
    check(lib().vg_select(ctx.h, ix.h, ctypes.byref(d), ctypes.byref(out), bu))
    return Relation(ctx, out), (bu[0], bu[1]) if bu[2] else None


def join(ctx: Context, l: Relation, r: Relation):
    out = vg_ir()
    fl = (ctypes.c_uint32 * 2)()
    check(lib().vg_join(ctx.h, ctypes.byref(l.ir), ctypes.byref(r.ir), ctypes.byref(out), fl))
    return Relation(ctx, out), (fl[0], fl[1])


def join2(ctx: Context, l: Relation, r: Relation):
    out = vg_ir()
    check(lib().vg_join2(ctx.h, ctypes.byref(l.ir), ctypes.byref(r.ir), ctypes.byref(out)))
    return Relation(ctx, out)


def swap(ctx: Context, rel: Relation, col: int) -> None:
    check(lib().vg_swap(ctx.h, ctypes.byref(rel.ir), col))


def sort_rows(ctx: Context, rel: Relation) -> None:
    check(lib().vg_sort_rows(ctx.h, ctypes.byref(rel.ir)))


def unique(ctx: Context, rel: Relation) -> None:
    check(lib().vg_unique(ctx.h, ctypes.byref(rel.ir)))


def eif_scan(ctx: Context, rel: Relation):
    out = (ctypes.c_uint64 * 4)()
    check(lib().vg_eif_scan(ctx.h, ctypes.byref(rel.ir), out))
    return tuple(out)


class Dict:
    """The loader's dictionaries (vg_dict): kind 0 subject/object, 1
    predicate, 2 literal; terms are their N-Triples text."""

    KINDS = {"so": 0, "p": 1, "l": 2}

    def __init__(self, handle):
        self.h = handle

    @staticmethod
    def open(path: str) -> "Dict":
        h = ctypes.c_void_p()
        check(lib().vg_dict_open(path.encode(), ctypes.byref(h)))
        return Dict(h)

    def write(self, path: str) -> None:
        check(lib().vg_dict_write(self.h, path.encode()))

    def size(self, kind) -> int:
        return int(lib().vg_dict_size(self.h, self.KINDS.get(kind, kind)))

    def term(self, kind, ident: int):
        t = lib().vg_dict_term(self.h, self.KINDS.get(kind, kind), ident)
        return None if t is None else t.decode("utf-8", "surrogateescape")

    def terms(self, kind) -> list:
        k = self.KINDS.get(kind, kind)
        base = 50000000 if k == 2 else 1
        return [self.term(k, base + i) for i in range(self.size(k))]

    def lookup(self, kind, term: str) -> int:
        return int(lib().vg_dict_lookup(self.h, self.KINDS.get(kind, kind), term.encode()))

    def close(self):
        if getattr(self, "h", None):
            lib().vg_dict_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ingested:
    """Device id columns from vg_ingest_ntriples and their dictionary."""

    def __init__(self, ctx, s, p, o, n, d):
        self.ctx, self.s, self.p, self.o, self.n, self.dict = ctx, s, p, o, n, d

    def device_ptrs(self):
        return [self.s, self.p, self.o]

    def index(self, full: bool = False) -> "Index":
        """Builds the permutation indexes straight from the device columns."""
        return Index(self.ctx, device_ptrs=self.device_ptrs(), n=self.n, full=full)

    def columns(self):
        """The three id columns copied to host arrays."""
        ir = vg_ir()
        ir.ncols, ir.nrows = 3, self.n
        for c, ptr in enumerate(self.device_ptrs()):
            ir.cols[c] = ptr
        out = []
        for c in range(3):
            a = np.zeros(self.n, dtype=np.uint32)
            if self.n:
                check(lib().vg_ir_download(self.ctx.h, ctypes.byref(ir), c, _p32(a)))
            out.append(a)
        return out

    def free(self):
        if self.s is not None:
            check(lib().vg_ingest_free(self.ctx.h, self.s, self.p, self.o))
            self.s = self.p = self.o = None


def ingest_ntriples(ctx: Context, text: bytes, literal_dict: bool = False) -> Ingested:
    """Parses N-Triples text on the device (vg_ingest_ntriples)."""
    s, p, o, d = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    n = ctypes.c_uint64()
    check(lib().vg_ingest_ntriples(ctx.h, text, len(text), int(literal_dict), ctypes.byref(s), ctypes.byref(p),
                                   ctypes.byref(o), ctypes.byref(n), ctypes.byref(d)))
    return Ingested(ctx, s.value, p.value, o.value, n.value, Dict(d))


def set_ingest_hash_bits(bits: int) -> None:
    lib().vg_ingest_set_hash_bits(bits)


def _decode(call) -> list:
    need = ctypes.c_size_t()
    st = call(None, 0, ctypes.byref(need))
    if st not in (0, 7):   # 7: VG_ERR_OVERFLOW, the size is in need
        check(st)
    buf = ctypes.create_string_buffer(need.value)
    check(call(buf, need.value, ctypes.byref(need)))
    text = buf.value.decode("utf-8", "surrogateescape")
    return [line.split("\t") for line in text.split("\n")[:-1]]


def decode_result(res: "Result", d: Dict) -> list:
    """Rows of a query result as terms (vg_result_decode)."""
    return _decode(lambda b, c, n: lib().vg_result_decode(res.h, d.h, b, c, n))


def decode_batch(batch: "Batch", q: int, d: Dict) -> list:
    """Rows of query q of a batch as terms (vg_batch_decode)."""
    return _decode(lambda b, c, n: lib().vg_batch_decode(batch.h, q, d.h, b, c, n))
