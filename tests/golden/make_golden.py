#!/usr/bin/env python
"""Generates the golden fixtures in this directory by running the reference
itself (oracle/_ref/vedas_ref: the reference's own sources compiled for the
host, see oracle/Makefile).  Needs the reference sources to build that binary;
the fixtures it writes are small JSON files that every other machine reads.

  python tests/golden/make_golden.py --ref-src /path/to/reference
  (or VEDAS_REF_SRC=/path/to/reference python tests/golden/make_golden.py)

Fixtures:
  index.json    sha256 and length of every index array (partial and full)
  queries.json  per query: status, headers, row count, sha256 of the rows in
                order, execution log -- on two small seeded graphs
  c1.json       the 1M-triple star query (?x p3 ?a . ?x p7 ?b)
  eid.json      the 22 updateBound vectors of the reference's
                test/TestDoubleBoundDict.cu (inputs, the test's expectations
                and what the reference code actually returns) plus random
                update sequences
  plans.json    plans the reference's QueryGraph builds for random estimates
  vds.json      the reference's own .vds files of a small graph
                (vds_partial.vds, vds_full.vds, written by VedasStorage::write)
                and their sha256
  plans_multiedge.json
                plans for random queries over few variables, with patterns that
                share both variables (several edges between two vertices) and
                equal estimates: the star-centre choice then falls to the
                iteration order of the reference's std::unordered_map

  python tests/golden/make_golden.py --only plans_multiedge   # one fixture
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_runner  # noqa: E402
from vedas_gb300 import workloads  # noqa: E402

INDEX_GRAPHS = {
    "star_small": dict(kind="star", n=20_000, n_subjects=1_500, seed=11),
    "chain_small": dict(kind="chain", n=30_000, n_entities=3_000, seed=12),
}
QUERY_GRAPHS = {
    "star_q": dict(kind="star", n=200_000, n_subjects=10_000, seed=21, nq=150, qseed=31),
    "chain_q": dict(kind="chain", n=300_000, n_entities=30_000, seed=22, nq=150, qseed=32),
}


def make_graph(spec):
    if spec["kind"] == "star":
        return workloads.graph_small_star(n=spec["n"], n_subjects=spec["n_subjects"], seed=spec["seed"])
    return workloads.graph_chain(n=spec["n"], n_entities=spec["n_entities"], seed=spec["seed"])


def digest_columns(cols) -> str:
    h = hashlib.sha256()
    for c in cols:
        h.update(np.ascontiguousarray(c, dtype=np.uint32).tobytes())
        h.update(b"|")
    return h.hexdigest()


def result_record(r) -> dict:
    rec = {"status": r.status, "headers": r.headers, "nrows": r.nrows,
           "sha256": digest_columns(r.columns) if r.status == "ok" else None,
           "log": [list(x[:4]) for x in r.log]}
    if r.status == "ok" and r.nrows <= 40:
        rec["rows"] = [c.tolist() for c in r.columns]
    return rec


def gen_index(td):
    out = {}
    for name, spec in INDEX_GRAPHS.items():
        g = make_graph(spec)
        p = os.path.join(td, name + ".graph")
        g.save(p)
        for full in (False, True):
            arrs = ref_runner.build_index(p, full=full)
            out[f"{name}/{'full' if full else 'partial'}"] = {
                k: {"len": int(v.shape[0]), "sha256": hashlib.sha256(v.tobytes()).hexdigest()}
                for k, v in arrs.items()}
    return {"graphs": INDEX_GRAPHS, "arrays": out}


VDS_GRAPH = dict(kind="star", n=3_000, n_subjects=300, seed=13)


def gen_vds(td):
    """The reference's own .vds files (VedasStorage::write) of a small graph,
    with the partial and the full index: vds_partial.vds, vds_full.vds."""
    g = make_graph(VDS_GRAPH)
    p = os.path.join(td, "vds.graph")
    g.save(p)
    files = {}
    for full in (False, True):
        name = f"vds_{'full' if full else 'partial'}.vds"
        out = os.path.join(HERE, name)
        # the full-index build writes histogram files into its working directory
        subprocess.run([ref_runner.REF_BIN, "vds-write", p, out] + (["full"] if full else []), check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, cwd=td)
        with open(out, "rb") as f:
            files[name] = hashlib.sha256(f.read()).hexdigest()
    return {"graph": VDS_GRAPH, "files": files}


def gen_queries(td):
    out = {}
    for name, spec in QUERY_GRAPHS.items():
        g = make_graph(spec)
        p = os.path.join(td, name + ".graph")
        g.save(p)
        qs = workloads.query_mix(g, spec["nq"], seed=spec["qseed"])
        res = ref_runner.run_queries(p, qs)
        out[name] = {"spec": spec, "queries": qs, "results": [result_record(r) for r in res]}
    return out


def gen_c1(td):
    g = workloads.graph_small_star()
    p = os.path.join(td, "c1.graph")
    g.save(p)
    q = workloads.star_query(3, 7)
    r = ref_runner.run_queries(p, [q])[0]
    return {"graph": "graph_small_star() defaults, seed 0", "query": q, "result": result_record(r)}


def parse_eid_tests(path):
    """The updateBound call sequences and testBound expectations of each TEST."""
    text = open(path).read()
    large = float(re.search(r"#define\s+LARGE_ID\s+([0-9eE.+]+)", text).group(1))
    cases = []
    for m in re.finditer(r"TEST\(EmptyIntervalDict,\s*(\w+)\)\s*\{(.*?)\n\}", text, re.S):
        name, body = m.group(1), m.group(2)

        def val(tok):
            tok = tok.strip()
            return int(large) if tok == "LARGE_ID" else int(float(tok))
        ups = [[val(x) for x in a.split(",")[1:]]
               for a in re.findall(r"updateBound\(([^)]*)\)", body)]
        exp = [val(x) for x in re.search(r"testBound\(bd,([^)]*)\)", body).group(1).split(",")]
        cases.append({"name": name, "updates": ups, "test_expects": exp})
    return cases


def run_eid(cases, td):
    inp = os.path.join(td, "eid.in")
    outp = os.path.join(td, "eid.out")
    with open(inp, "w") as f:
        for c in cases:
            f.write("reset\n")
            for u in c["updates"]:
                f.write("update " + " ".join(str(x) for x in u) + "\n")
            f.write("get\n")
    subprocess.run([ref_runner.REF_BIN, "eid", inp, outp], check=True)
    lines = open(outp).read().split("\n")
    for c, ln in zip(cases, lines):
        c["reference"] = [int(x) for x in ln.split()]
    return cases


def gen_eid(ref_src, td):
    cases = parse_eid_tests(os.path.join(ref_src, "test", "TestDoubleBoundDict.cu"))
    rng = np.random.Generator(np.random.PCG64(41))
    rand = []
    for i in range(300):
        ups = []
        for _ in range(int(rng.integers(1, 5))):
            u = [int(x) for x in rng.integers(0, 60, size=4)]
            if rng.random() < 0.15:
                u[int(rng.integers(0, 4))] = 4294967295
            if rng.random() < 0.2:
                u[0] = u[1] = 0
            ups.append(u)
        rand.append({"name": f"random{i}", "updates": ups})
    return {"test_file": run_eid(cases, td), "random": run_eid(rand, td)}


def gen_plans(td):
    g = workloads.graph_small_star(n=20_000, n_subjects=1_500, seed=51)
    cs = workloads.ConstantSampler(g)
    rng = np.random.Generator(np.random.PCG64(52))
    cases = []
    for i in range(400):
        q = workloads.instantiate(workloads.TEMPLATES[i % len(workloads.TEMPLATES)][1], cs, rng)
        npat = q.count(" . ") + 1
        if rng.random() < 0.5:
            est = [int(x) for x in rng.integers(0, 3, size=npat) * 1000]   # many ties
        else:
            est = [int(x) for x in rng.integers(0, 100_000, size=npat)]
        cases.append({"query": q, "estimates": est})
    inp = os.path.join(td, "plan.in")
    outp = os.path.join(td, "plan.out")
    with open(inp, "w") as f:
        for c in cases:
            f.write(" ".join(str(e) for e in c["estimates"]) + "|" + c["query"] + "\n")
    subprocess.run([ref_runner.REF_BIN, "plan", inp, outp], check=True)
    for c, ln in zip(cases, open(outp).read().split("\n")):
        c["reference_plan"] = ln
    return cases


def gen_plans_multiedge(td):
    """Random basic graph patterns over two to four variables, so that
    patterns often share both of their variables, with estimates drawn from
    {5, 7, 1000} (ties).  Queries on which the reference's planner loops
    forever (a star step that merges nothing) are left out: the oracle's
    planner reports them, and the reference run is bounded by a timeout."""
    import ctypes
    from oracle import oracle_py
    O = oracle_py.lib()
    O.vo_plan_describe.restype = ctypes.c_int
    O.vo_plan_describe.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32,
                                   ctypes.c_char_p, ctypes.c_uint64]
    rng = np.random.Generator(np.random.PCG64(61))
    names = ["?a", "?b", "?c", "?d"]
    cases = []
    while len(cases) < 300:
        npat = int(rng.integers(2, 6))
        pats = []
        for _ in range(npat):
            nv = int(rng.integers(2, 5))
            s, o = rng.choice(names[:nv], size=2, replace=False)
            pats.append(f"{s} <{int(rng.integers(1, 10))}> {o}")
        q = "SELECT * WHERE { " + " . ".join(pats) + " . }"
        est = [int(x) for x in rng.choice([5, 5, 7, 1000], size=npat)]
        e = np.array(est, dtype=np.uint64)
        buf = ctypes.create_string_buffer(8192)
        if O.vo_plan_describe(q.encode(), e.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(est), buf,
                              8192) == 0:
            cases.append({"query": q, "estimates": est})
    inp = os.path.join(td, "plan_me.in")
    outp = os.path.join(td, "plan_me.out")
    with open(inp, "w") as f:
        for c in cases:
            f.write(" ".join(str(x) for x in c["estimates"]) + "|" + c["query"] + "\n")
    subprocess.run([ref_runner.REF_BIN, "plan", inp, outp], check=True, timeout=120)
    for c, ln in zip(cases, open(outp).read().split("\n")):
        c["reference_plan"] = ln
    return cases


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=os.environ.get("VEDAS_REF_SRC"),
                    help="the reference checkout (default: $VEDAS_REF_SRC; required)")
    ap.add_argument("--only", default=None, help="write only this fixture (its file name without .json)")
    a = ap.parse_args()
    if not a.ref_src:
        ap.error("give the reference checkout with --ref-src or VEDAS_REF_SRC")
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={a.ref_src}"],
                   check=True)
    with tempfile.TemporaryDirectory() as td:
        for name, fn in (("index", lambda: gen_index(td)), ("queries", lambda: gen_queries(td)),
                         ("c1", lambda: gen_c1(td)), ("eid", lambda: gen_eid(a.ref_src, td)),
                         ("plans", lambda: gen_plans(td)),
                         ("plans_multiedge", lambda: gen_plans_multiedge(td)),
                         ("vds", lambda: gen_vds(td))):
            if a.only and name != a.only:
                continue
            data = fn()
            with open(os.path.join(HERE, name + ".json"), "w") as f:
                json.dump(data, f, separators=(",", ":"))
            print("wrote", name)


if __name__ == "__main__":
    main()
