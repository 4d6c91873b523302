"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker, never by the product package.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u64, u32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32
        pu32 = ctypes.POINTER(ctypes.c_uint32)
        L.vo_index_build.restype = vp
        L.vo_index_build.argtypes = [pu32, pu32, pu32, u64, ctypes.c_int]
        L.vo_index_free.argtypes = [vp]
        L.vo_index_array.restype = ctypes.c_int
        L.vo_index_array.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(pu32),
                                     ctypes.POINTER(u64)]
        L.vo_query.restype = vp
        L.vo_query.argtypes = [vp, ctypes.c_char_p]
        L.vo_result_status.restype = ctypes.c_int
        L.vo_result_status.argtypes = [vp]
        L.vo_result_error.restype = ctypes.c_char_p
        L.vo_result_error.argtypes = [vp]
        L.vo_result_ncols.restype = u32
        L.vo_result_ncols.argtypes = [vp]
        L.vo_result_header.restype = ctypes.c_char_p
        L.vo_result_header.argtypes = [vp, u32]
        L.vo_result_nrows.restype = u64
        L.vo_result_nrows.argtypes = [vp]
        L.vo_result_column.restype = pu32
        L.vo_result_column.argtypes = [vp, u32]
        L.vo_result_nlog.restype = u32
        L.vo_result_nlog.argtypes = [vp]
        L.vo_result_log.argtypes = [vp, u32, ctypes.POINTER(u32), ctypes.POINTER(u64),
                                    ctypes.POINTER(u64), ctypes.POINTER(u64),
                                    ctypes.POINTER(ctypes.c_char_p)]
        L.vo_result_free.argtypes = [vp]
        L.vo_sort_by_first.argtypes = [ctypes.POINTER(pu32), u32, u64]
        L.vo_inner_join.restype = u64
        L.vo_inner_join.argtypes = [pu32, u64, pu32, u64, ctypes.POINTER(u64),
                                    ctypes.POINTER(u64)]
        L.vo_ingest_ntriples.restype = u64
        L.vo_ingest_ntriples.argtypes = [ctypes.c_char_p, u64, ctypes.c_int, ctypes.POINTER(u64),
                                         ctypes.POINTER(pu32), ctypes.POINTER(pu32), ctypes.POINTER(pu32),
                                         ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
        L.vo_free.argtypes = [vp]
        _lib = L
    return _lib


def _p32(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


OPS = {0: "JOIN", 1: "UPLOAD", 2: "SWAP"}


@dataclasses.dataclass
class Result:
    status: int
    error: str
    headers: list
    columns: list
    log: list

    @property
    def nrows(self) -> int:
        return int(self.columns[0].shape[0]) if self.columns else 0


class OracleIndex:
    """The reference index layout built on the CPU, plus the query path."""

    def __init__(self, s, p, o, full: bool = False):
        L = lib()
        self._keep = [np.ascontiguousarray(x, dtype=np.uint32) for x in (s, p, o)]
        self.h = L.vo_index_build(_p32(self._keep[0]), _p32(self._keep[1]),
                                  _p32(self._keep[2]), len(self._keep[0]), int(full))

    def __del__(self):
        if getattr(self, "h", None):
            lib().vo_index_free(self.h)
            self.h = None

    def array(self, name: str) -> np.ndarray:
        ptr = ctypes.POINTER(ctypes.c_uint32)()
        n = ctypes.c_uint64()
        if lib().vo_index_array(self.h, name.encode(), ctypes.byref(ptr), ctypes.byref(n)):
            raise KeyError(name)
        if n.value == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.ctypeslib.as_array(ptr, shape=(n.value,)).copy()

    def query(self, text: str) -> Result:
        L = lib()
        r = L.vo_query(self.h, text.encode())
        try:
            st = L.vo_result_status(r)
            err = L.vo_result_error(r).decode()
            heads, cols = [], []
            if st == 0:
                nr = L.vo_result_nrows(r)
                for c in range(L.vo_result_ncols(r)):
                    heads.append(L.vo_result_header(r, c).decode())
                    if nr:
                        cols.append(np.ctypeslib.as_array(L.vo_result_column(r, c),
                                                          shape=(nr,)).copy())
                    else:
                        cols.append(np.zeros(0, dtype=np.uint32))
            log = []
            for i in range(L.vo_result_nlog(r)):
                op, p1, p2, p3 = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
                txt = ctypes.c_char_p()
                L.vo_result_log(r, i, ctypes.byref(op), ctypes.byref(p1), ctypes.byref(p2),
                                ctypes.byref(p3), ctypes.byref(txt))
                log.append((OPS[op.value], p1.value, p2.value, p3.value, txt.value.decode()))
            return Result(st, err, heads, cols, log)
        finally:
            L.vo_result_free(r)


def sort_by_first(cols):
    """Stable sort of the rows of `cols` (list of uint32 arrays) by column 0."""
    cols = [np.ascontiguousarray(c, dtype=np.uint32).copy() for c in cols]
    arr = (ctypes.POINTER(ctypes.c_uint32) * len(cols))(*[_p32(c) for c in cols])
    lib().vo_sort_by_first(arr, len(cols), cols[0].shape[0] if cols else 0)
    return cols


def inner_join(a, b):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    n = lib().vo_inner_join(_p32(a), len(a), _p32(b), len(b), None, None)
    li = np.zeros(n, dtype=np.uint64)
    ri = np.zeros(n, dtype=np.uint64)
    lib().vo_inner_join(_p32(a), len(a), _p32(b), len(b),
                        li.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                        ri.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return li, ri


def ingest_ntriples(text: bytes, literal_dict: bool = False):
    """(s, p, o, {"so": [...], "p": [...], "l": [...]}) as the reference's
    loader assigns them (src/loader.cu:19-53); raises ValueError with the
    line number of a malformed statement."""
    L = lib()
    pu32 = ctypes.POINTER(ctypes.c_uint32)
    n = ctypes.c_uint64()
    s, p, o = pu32(), pu32(), pu32()
    ts = [ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()]
    bad = L.vo_ingest_ntriples(text, len(text), int(literal_dict), ctypes.byref(n), ctypes.byref(s),
                               ctypes.byref(p), ctypes.byref(o), ctypes.byref(ts[0]), ctypes.byref(ts[1]),
                               ctypes.byref(ts[2]))
    if bad:
        raise ValueError(f"malformed N-Triples statement on line {bad}")
    cols = []
    for c in (s, p, o):
        cols.append(np.ctypeslib.as_array(c, shape=(max(n.value, 1),))[:n.value].copy())
        L.vo_free(ctypes.cast(c, ctypes.c_void_p))
    dicts = {}
    for name, t in zip(("so", "p", "l"), ts):
        raw = ctypes.string_at(t.value).decode("utf-8", "surrogateescape")
        dicts[name] = raw.split("\n")[:-1] if raw else []
        L.vo_free(t)
    return cols[0], cols[1], cols[2], dicts
