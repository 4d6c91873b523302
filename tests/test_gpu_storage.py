"""The .vds index file (VedasStorage::write / open, src/VedasStorage.cu:459-516)
against the reference's own files: tests/golden/vds_partial.vds and
vds_full.vds were written by the reference (tests/golden/make_golden.py).
The core opens them into arrays equal to the oracle's and answers queries
on them as on a built index; the files the core writes for the same graph
are byte for byte the reference's, so the reference opens them too."""
import json
import os

import numpy as np
import pytest

from oracle import oracle_py
from vedas_gb300 import workloads

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARTIAL = ["p_idx_values", "p_idx_offsets", "ps_s_idx_values", "ps_idx_offsets", "po_o_idx_values",
           "po_idx_offsets", "ps_data", "po_data", "pso_data", "pos_data"]
FULL = ["s_idx_values", "s_idx_offsets", "sp_p_idx_values", "sp_idx_offsets", "so_o_idx_values",
        "so_idx_offsets", "o_idx_values", "o_idx_offsets", "os_data", "op_p_idx_values", "op_idx_offsets",
        "spo_data", "sop_data", "ops_data", "osp_data"]


def _graph():
    spec = json.load(open(os.path.join(GOLDEN, "vds.json")))["graph"]
    return workloads.graph_small_star(n=spec["n"], n_subjects=spec["n_subjects"], seed=spec["seed"])


@pytest.mark.parametrize("full", [False, True])
def test_reference_vds_opens_and_core_writes_the_same_bytes(ctx, tmp_path, full):
    import vedas_gb300 as vg
    g = _graph()
    name = f"vds_{'full' if full else 'partial'}.vds"
    ref_path = os.path.join(GOLDEN, name)
    ox = oracle_py.OracleIndex(g.s, g.p, g.o, full=full)
    opened = vg.Index.open(ctx, ref_path, full=full)
    for a in PARTIAL + (FULL if full else []):
        np.testing.assert_array_equal(opened.array(a), ox.array(a), err_msg=a)
    # queries on the opened index equal the oracle's
    qs = workloads.query_mix(g, 60, seed=5)
    for q in qs:
        r = ox.query(q)
        if r.status != 0:
            continue
        res = opened.query(q)
        assert res.headers == r.headers
        for x, y in zip(res.columns(), r.columns):
            np.testing.assert_array_equal(x, y)
        res.close()
    # the core's own file of the same graph is the reference's, byte for byte
    built = vg.Index(ctx, g.s, g.p, g.o, full=full)
    out = str(tmp_path / name)
    built.write(out)
    assert open(out, "rb").read() == open(ref_path, "rb").read()
    # and a file the core wrote opens again with the same arrays
    again = vg.Index.open(ctx, out, full=full)
    for a in PARTIAL + (FULL if full else []):
        np.testing.assert_array_equal(again.array(a), ox.array(a), err_msg=a)
    for ix in (opened, built, again):
        ix.close()
