"""Runs the reference-as-oracle binary (oracle/_ref/vedas_ref) from Python.

Test infrastructure only.  The binary is the VEDAS reference's own source
compiled for the host (see oracle/Makefile); it exists only where the
reference sources were available to build it.  Results are parsed into
``RefResult`` records; a query that makes the reference abort (its asserts
are live) is reported with ``status == "abort"`` and the runner resumes at
the next query.
"""
from __future__ import annotations

import dataclasses
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "vedas_ref")

OPS = {0: "JOIN", 1: "UPLOAD", 2: "SWAP"}


def available() -> bool:
    return os.path.exists(REF_BIN)


@dataclasses.dataclass
class RefResult:
    index: int
    status: str                      # "ok" | "abort" | "empty"
    headers: list
    columns: list                    # list of np.uint32 arrays
    log: list                        # (op, p1, p2, p3, text)

    @property
    def nrows(self) -> int:
        return int(self.columns[0].shape[0]) if self.columns else 0


def _read_str(buf, off):
    (ln,) = struct.unpack_from("<I", buf, off)
    off += 4
    return buf[off:off + ln].decode(), off + ln


def parse_results(buf: bytes):
    out = []
    off = 0
    while off < len(buf):
        qi, empty, ncols = struct.unpack_from("<III", buf, off)
        off += 12
        (nrows,) = struct.unpack_from("<Q", buf, off)
        off += 8
        headers, cols = [], []
        for _ in range(ncols):
            h, off = _read_str(buf, off)
            headers.append(h)
            cols.append(np.frombuffer(buf, dtype=np.uint32, count=nrows, offset=off).copy())
            off += 4 * nrows
        (nlog,) = struct.unpack_from("<I", buf, off)
        off += 4
        log = []
        for _ in range(nlog):
            (op,) = struct.unpack_from("<I", buf, off)
            p1, p2, p3 = struct.unpack_from("<QQQ", buf, off + 4)
            off += 28
            txt, off = _read_str(buf, off)
            log.append((OPS.get(op, str(op)), p1, p2, p3, txt))
        out.append(RefResult(qi, "empty" if empty else "ok", headers, cols, log))
    return out


def parse_index(buf: bytes) -> dict:
    arrs = {}
    off = 0
    while True:
        name, off = _read_str(buf, off)
        if not name:
            break
        (n,) = struct.unpack_from("<Q", buf, off)
        off += 8
        arrs[name] = np.frombuffer(buf, dtype=np.uint32, count=n, offset=off).copy()
        off += 4 * n
    return arrs


def build_index(graph_path: str, full: bool = False) -> dict:
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "idx.bin")
        cmd = [REF_BIN, "index", os.path.abspath(graph_path), out] + (["full"] if full else [])
        # the reference's full-index build writes histogram files into its
        # working directory (VedasStorage::writeHistogram): keep them in td
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, cwd=td)
        with open(out, "rb") as f:
            return parse_index(f.read())


def run_queries(graph_path: str, queries: list, full: bool = False, timeout: float = 600.0):
    """Runs every query through the reference; returns one RefResult per query."""
    results = {}
    with tempfile.TemporaryDirectory() as td:
        qpath = os.path.join(td, "q.txt")
        with open(qpath, "w") as f:
            for q in queries:
                f.write(q.replace("\n", " ") + "\n")
        out = os.path.join(td, "res.bin")
        first = 0
        while first < len(queries):
            cmd = [REF_BIN, "query", os.path.abspath(graph_path), qpath, out, str(first)] + \
                (["full"] if full else [])
            proc = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                                  timeout=timeout, cwd=td)
            with open(out, "rb") as f:
                parsed = parse_results(f.read())
            for r in parsed:
                results[r.index] = r
            done = max(results) + 1 if results else 0
            if proc.returncode == 0 and done >= len(queries):
                break
            # the query at `done` aborted the reference: record it, go on
            results[done] = RefResult(done, "abort", [], [], [])
            first = done + 1
    return [results[i] for i in range(len(queries))]
